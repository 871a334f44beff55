// Host side of the C-ABI in include/tcs.h: argument checks, tensor-map
// encoding, plans (device state + captured multi-step graphs), the one-call
// host form, and the drop-in replacements of the reference's host_code.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "batch.h"
#include "tcs_internal.h"

namespace tcs {

namespace {
thread_local std::string t_last_error;
}

int fail(int status, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return status;
}

int cuda_status(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return TCS_OK;
    return fail(e == cudaErrorMemoryAllocation ? TCS_ERR_NOMEM : TCS_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

int make_geom(int ny, int nx, int stencil, int y0, int y1, int x0, int x1, GridGeom *geom) {
    if (stencil < TCS_STAR2D1R || stencil > TCS_BOX2D2R)
        return fail(TCS_ERR_INVALID, "unknown stencil %d", stencil);
    const int r = stencil_r(stencil);
    if (ny < 2 * r + 1 || nx < 2 * r + 1 || ny > (1 << 24) || nx > (1 << 24))
        return fail(TCS_ERR_INVALID, "grid %d x %d out of range for radius %d", ny, nx, r);
    if (y0 == 0 && y1 == 0 && x0 == 0 && x1 == 0) {
        y0 = r; y1 = ny - r; x0 = r; x1 = nx - r;
    }
    if (y0 < r || x0 < r || y1 > ny - r || x1 > nx - r || y0 > y1 || x0 > x1)
        return fail(TCS_ERR_INVALID,
                    "update rectangle [%d,%d) x [%d,%d) must lie inside [%d,%d) x [%d,%d)", y0, y1,
                    x0, x1, r, ny - r, r, nx - r);
    geom->ny = ny;
    geom->nx = nx;
    geom->y0 = y0; geom->y1 = y1; geom->x0 = x0; geom->x1 = x1;
    geom->p16 = plane_geom(ny, nx, 8);
    geom->p32 = plane_geom(ny, nx, 4);
    return TCS_OK;
}

TapCoeffs tap_coeffs(int stencil, const float *B) {
    TapCoeffs c;
    const int r = stencil_r(stencil), n = 2 * r + 1;
    for (int k = 0; k < 25; k++) c.c[k] = 0.0f;
    for (int k = 0; k < tap_count(stencil); k++)
        c.c[k] = B[(tap_dy(stencil, k) + r) * n + tap_dx(stencil, k) + r];
    return c;
}

double tap_abs_sum(int stencil, const float *B) {
    const TapCoeffs c = tap_coeffs(stencil, B);
    double s = 0.0;
    for (int k = 0; k < tap_count(stencil); k++) s += std::fabs((double)c.c[k]);
    return s;
}

int split_scale_exp(float max_abs) {
    if (!(max_abs > 0.0f) || !std::isfinite(max_abs)) return 0;
    int e = 0;
    const float m = std::frexp(max_abs, &e);  // max_abs = m 2^e, m in [0.5, 1)
    (void)m;
    return e;  // max_abs < 2^e, so max_abs 2^-e < 1
}

// --------------------------------------------------------- one sweep step --
namespace {

// The split form keeps its fixed-point hi plane exact only for stencils that
// do not expand the data (sum of |c| <= 1, with slack for FP32 rounding of a
// normalised set).
int check_split_coeffs(int stencil, int precision, const float *B) {
    if (precision != TCS_PREC_SPLIT) return TCS_OK;
    const double s = tap_abs_sum(stencil, B);
    if (!(s <= kSplitMaxAbsSum))
        return fail(TCS_ERR_UNSUPPORTED,
                    "split precision needs a non-expanding stencil (sum of |c| <= 1), got %g", s);
    return TCS_OK;
}

int check_mode(int engine, int precision) {
    if (engine != TCS_ENGINE_TENSOR && engine != TCS_ENGINE_CUDACORE)
        return fail(TCS_ERR_INVALID, "unknown engine %d", engine);
    if (precision < TCS_PREC_F16 || precision > TCS_PREC_F32)
        return fail(TCS_ERR_INVALID, "unknown precision %d", precision);
    if (engine == TCS_ENGINE_TENSOR && precision == TCS_PREC_F32)
        return fail(TCS_ERR_UNSUPPORTED, "FP32 storage runs on the CUDA-core engine only");
    if (engine == TCS_ENGINE_CUDACORE && precision == TCS_PREC_SPLIT)
        return fail(TCS_ERR_UNSUPPORTED, "split precision runs on the tensor engine only");
    return TCS_OK;
}

// One step from the input planes to the output planes.
int run_step(const GridGeom &g, int stencil, int engine, int precision, const float *B,
             const void *in, const void *in_lo, void *out, void *out_lo, cudaStream_t s,
             int tile_w = kTile, SplitScale *scale = nullptr, int t0 = 0) {
    cudaError_t e;
    if (engine == TCS_ENGINE_CUDACORE) {
        const TapCoeffs c = tap_coeffs(stencil, B);
        if (precision == TCS_PREC_F32)
            e = launch_cc_f32(g, stencil, c, static_cast<const float *>(in),
                              static_cast<float *>(out), s);
        else
            e = launch_cc_f16(g, stencil, c, static_cast<const uint16_t *>(in),
                              static_cast<uint16_t *>(out), s);
    } else if (precision == TCS_PREC_SPLIT) {
        e = launch_tc_split(g, stencil, B, static_cast<const uint16_t *>(in),
                            static_cast<const uint16_t *>(in_lo), static_cast<uint16_t *>(out),
                            static_cast<uint16_t *>(out_lo), s, scale, t0);
    } else {
        e = launch_tc_f16(g, stencil, B, static_cast<const uint16_t *>(in),
                          static_cast<uint16_t *>(out), s, tile_w);
    }
    return cuda_status(e, "sweep kernel launch");
}

}  // namespace

}  // namespace tcs

using namespace tcs;

// ================================================================ C-ABI ==
extern "C" {

const char *tcs_status_string(int status) {
    switch (status) {
    case TCS_OK: return "ok";
    case TCS_ERR_INVALID: return "invalid argument";
    case TCS_ERR_CUDA: return "CUDA error";
    case TCS_ERR_UNSUPPORTED: return "unsupported";
    case TCS_ERR_NOMEM: return "out of device memory";
    case TCS_ERR_TIMEOUT: return "device wait timed out";
    case TCS_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
    }
}

const char *tcs_last_error(void) { return t_last_error.c_str(); }

int tcs_stencil_radius(int stencil) {
    return (stencil < TCS_STAR2D1R || stencil > TCS_BOX2D2R) ? -1 : stencil_r(stencil);
}

size_t tcs_brick_elems(int ny, int nx) {
    if (ny <= 0 || nx <= 0) return 0;
    return (size_t)((ny + 15) / 16) * (size_t)((nx + 15) / 16) * 256;
}

size_t tcs_plane_elems(int ny, int nx, int precision) {
    if (ny <= 0 || nx <= 0 || precision < TCS_PREC_F16 || precision > TCS_PREC_F32) return 0;
    return plane_elems(plane_geom(ny, nx, precision == TCS_PREC_F32 ? 4 : 8));
}

int tcs_device_error(int *code) {
    int st = cuda_status(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (st) return st;
    int c = 0;
    st = cuda_status(tc_take_error(&c), "reading the device error word");
    if (st) return st;
    int cb = 0;
    st = cuda_status(batch_take_error(&cb), "reading the batch error word");
    if (st) return st;
    if (!c) c = cb;
    st = cuda_status(tb_take_error(&cb), "reading the blocked-sweep error word");
    if (st) return st;
    if (!c) c = cb;
    st = cuda_status(cc_take_error(&cb), "reading the CUDA-core error word");
    if (st) return st;
    if (!c) c = cb;
    if (code) *code = c;
    return c ? fail(TCS_ERR_TIMEOUT, "device wait timed out (code %d)", c) : TCS_OK;
}

// ----------------------------------------------------- layout transforms --
int tcs_padding_2d(const uint16_t *d_in, uint16_t *d_out, int size, int halo, uint16_t value16,
                   void *stream) {
    if (!d_in || !d_out || size <= 0 || halo < 0) return fail(TCS_ERR_INVALID, "tcs_padding_2d: bad arguments");
    return cuda_status(launch_padding_2d(d_in, d_out, size, halo, value16, (cudaStream_t)stream),
                       "padding_2d launch");
}

int tcs_brick_layout_2d(const uint16_t *d_in, uint16_t *d_out, int ny, int nx, void *stream) {
    if (!d_in || !d_out || ny <= 0 || nx <= 0) return fail(TCS_ERR_INVALID, "tcs_brick_layout_2d: bad arguments");
    return cuda_status(launch_brick_2d(d_in, d_out, ny, nx, (cudaStream_t)stream), "brick_2d launch");
}

int tcs_reverse_layout_2d(const uint16_t *d_in, uint16_t *d_out, int ny, int nx, void *stream) {
    if (!d_in || !d_out || ny <= 0 || nx <= 0) return fail(TCS_ERR_INVALID, "tcs_reverse_layout_2d: bad arguments");
    return cuda_status(launch_unbrick_2d(d_in, d_out, ny, nx, (cudaStream_t)stream), "unbrick_2d launch");
}

#define TCS_CHECK_PACK(name)                                                        \
    if (!d_in || ny <= 0 || nx <= 0 || pad < 0) return fail(TCS_ERR_INVALID, name ": bad arguments")

int tcs_pack_f16(const float *d_in, int ny, int nx, int pad, float pad_value, uint16_t *d_bricks,
                 void *stream) {
    TCS_CHECK_PACK("tcs_pack_f16");
    return cuda_status(launch_pack_f16(d_in, ny, nx, pad, pad_value, d_bricks, (cudaStream_t)stream), "pack_f16 launch");
}
int tcs_unpack_f16(const uint16_t *d_in, int ny, int nx, int pad, float *d_out, void *stream) {
    TCS_CHECK_PACK("tcs_unpack_f16");
    return cuda_status(launch_unpack_f16(d_in, ny, nx, pad, d_out, (cudaStream_t)stream), "unpack_f16 launch");
}
int tcs_pack_f32(const float *d_in, int ny, int nx, int pad, float pad_value, float *d_bricks,
                 void *stream) {
    TCS_CHECK_PACK("tcs_pack_f32");
    return cuda_status(launch_pack_f32(d_in, ny, nx, pad, pad_value, d_bricks, (cudaStream_t)stream), "pack_f32 launch");
}
int tcs_unpack_f32(const float *d_in, int ny, int nx, int pad, float *d_out, void *stream) {
    TCS_CHECK_PACK("tcs_unpack_f32");
    return cuda_status(launch_unpack_f32(d_in, ny, nx, pad, d_out, (cudaStream_t)stream), "unpack_f32 launch");
}
int tcs_pack_split(const float *d_in, int ny, int nx, int pad, float pad_value, int scale_exp,
                   uint16_t *d_hi, uint16_t *d_lo, void *stream) {
    TCS_CHECK_PACK("tcs_pack_split");
    return cuda_status(launch_pack_split(d_in, ny, nx, pad, pad_value, scale_exp, d_hi, d_lo, (cudaStream_t)stream), "pack_split launch");
}
int tcs_max_abs_f32(const float *d_in, size_t n, float *h_max, void *stream) {
    if (!d_in || !h_max) return fail(TCS_ERR_INVALID, "tcs_max_abs_f32: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned *d = nullptr, bits = 0;
    int st = dev_alloc_t(&d, sizeof(unsigned), "max");
    if (!st) st = cuda_status(cudaMemsetAsync(d, 0, sizeof(unsigned), s), "memset(max)");
    if (!st) st = cuda_status(launch_max_abs(d_in, n, d, s), "max_abs launch");
    if (!st) st = cuda_status(cudaMemcpyAsync(&bits, d, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "max copy");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (d) dev_free(d);
    if (!st) std::memcpy(h_max, &bits, sizeof(float));
    return st;
}

int tcs_split_scale_exp(float max_abs) { return split_scale_exp(max_abs); }

int tcs_unpack_split(const uint16_t *d_hi, const uint16_t *d_lo, int ny, int nx, int pad,
                     int scale_exp, float *d_out, void *stream) {
    const void *d_in = d_hi;
    TCS_CHECK_PACK("tcs_unpack_split");
    return cuda_status(launch_unpack_split(d_hi, d_lo, ny, nx, pad, scale_exp, d_out, (cudaStream_t)stream), "unpack_split launch");
}

// ---------------------------------------------------------- band builders --
// init_coe of layout16/host_star2d1r.cu:33-61 and host_star2d2r.cu:33-67:
// vertical band `a` (row i+r holds taps at columns i..i+2r) and horizontal
// band `b` (column i+r holds taps at rows i..i+2r, centre tap zeroed), with
// the rows/columns that run past the brick edge clipped.
int tcs_init_coe_star(const uint16_t *B16, int n, uint16_t *a, uint16_t *b) {
    if (!B16 || !a || !b || (n != 3 && n != 5)) return fail(TCS_ERR_INVALID, "tcs_init_coe_star: bad arguments");
    const int r = n / 2;
    uint16_t vert[5], hori[5];
    for (int i = 0; i < n; i++) {
        hori[i] = B16[r * n + i];
        vert[i] = B16[r + i * n];
    }
    hori[r] = 0;
    std::memset(a, 0, 256 * sizeof(uint16_t));
    std::memset(b, 0, 256 * sizeof(uint16_t));
    for (int row = 0; row < 16; row++)
        for (int j = 0; j < n; j++) {
            const int col = row - r + j;  // band entry (row, col) = tap j
            if (col < 0 || col > 15) continue;
            a[row * 16 + col] = vert[j];
            b[col * 16 + row] = hori[j];
        }
    return TCS_OK;
}

// init_coe of layout16/host_box2d1r.cu:29-46 and host_box2d2r.cu:29-50: band
// z is the horizontal band of coefficient row z, clipped at the brick edge.
int tcs_init_coe_box(const uint16_t *B16, int n, uint16_t *coe) {
    if (!B16 || !coe || (n != 3 && n != 5)) return fail(TCS_ERR_INVALID, "tcs_init_coe_box: bad arguments");
    const int r = n / 2;
    std::memset(coe, 0, (size_t)256 * n * sizeof(uint16_t));
    for (int z = 0; z < n; z++)
        for (int col = 0; col < 16; col++)
            for (int j = 0; j < n; j++) {
                const int row = col - r + j;
                if (row < 0 || row > 15) continue;
                coe[z * 256 + row * 16 + col] = B16[z * n + j];
            }
    return TCS_OK;
}

// ------------------------------------------------------------------ step --
int tcs_sweep_step(const tcs_step_args *a, const void *d_in, const void *d_in_lo, void *d_out,
                   void *d_out_lo, void *stream) {
    if (!a || !a->coeffs || !d_in || !d_out) return fail(TCS_ERR_INVALID, "tcs_sweep_step: null argument");
    if (d_in == d_out) return fail(TCS_ERR_INVALID, "tcs_sweep_step: input and output must differ");
    int st = check_mode(a->engine, a->precision);
    if (st) return st;
    if (a->precision == TCS_PREC_SPLIT && (!d_in_lo || !d_out_lo))
        return fail(TCS_ERR_INVALID, "tcs_sweep_step: split precision needs lo planes");
    if (a->stencil < TCS_STAR2D1R || a->stencil > TCS_BOX2D2R)
        return fail(TCS_ERR_INVALID, "unknown stencil %d", a->stencil);
    st = check_split_coeffs(a->stencil, a->precision, a->coeffs);
    if (st) return st;
    GridGeom g;
    st = make_geom(a->ny, a->nx, a->stencil, a->y0, a->y1, a->x0, a->x1, &g);
    if (st) return st;
    if (reinterpret_cast<uintptr_t>(d_in) % 16 || reinterpret_cast<uintptr_t>(d_out) % 16 ||
        reinterpret_cast<uintptr_t>(d_in_lo) % 16 || reinterpret_cast<uintptr_t>(d_out_lo) % 16)
        return fail(TCS_ERR_INVALID, "tcs_sweep_step: planes must be 16-byte aligned");
    if (a->engine == TCS_ENGINE_TENSOR) {
        st = cuda_status(tc_prepare(a->stencil, a->precision == TCS_PREC_SPLIT), "tensor kernel set-up");
        if (st) return st;
    }
    return run_step(g, a->stencil, a->engine, a->precision, a->coeffs, d_in, d_in_lo, d_out,
                    d_out_lo, (cudaStream_t)stream);
}

}  // extern "C"

// ================================================================= plans ==
namespace {

// SM count of the device (read once).
int device_sms() {
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

}  // namespace

struct tcs_plan_s {
    tcs_problem prob;
    float coeffs[25];
    GridGeom g;
    size_t plane_bytes = 0;
    void *buf[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [state][hi, lo]
    int cur = 0;
    SplitScale *d_scale = nullptr;  // split form: per-step scale; the planes hold x 2^-E
    unsigned *d_max = nullptr;      // split form: max |x| scratch (float bits)
    float *staging = nullptr;   // ny*nx FP32, for host/row-major transfers
    // host transfers in row bands: packing (unpacking) of one band on `aux`
    // while the next band's copy runs on the caller's stream
    static constexpr int kBands = 4;
    cudaStream_t aux = nullptr;
    cudaEvent_t band_ev[kBands + 1] = {};
    cudaStream_t capture_stream = nullptr;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (steps, start state)
    unsigned *rows_done = nullptr;  // plain tensor form: per tile row, for multi-step launches

    int planes() const { return prob.precision == TCS_PREC_SPLIT ? 2 : 1; }

    void drop_graphs() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    ~tcs_plan_s() {
        drop_graphs();
        for (auto &s : buf)
            for (auto &p : s)
                if (p) dev_free(p);
        if (staging) dev_free(staging);
        if (d_max) dev_free(d_max);
        if (d_scale) dev_free(d_scale);
        if (rows_done) dev_free(rows_done);
        for (cudaEvent_t e : band_ev)
            if (e) cudaEventDestroy(e);
        if (aux) cudaStreamDestroy(aux);
        if (capture_stream) cudaStreamDestroy(capture_stream);
    }

    // FP16 and FP32 grids of at least 8 MB move in bands; split grids need
    // their maximum before packing, and small ones gain nothing.
    bool banded() const {
        return prob.precision != TCS_PREC_SPLIT &&
               (size_t)prob.ny * prob.nx * sizeof(float) >= ((size_t)8 << 20);
    }
    int ensure_bands() {
        if (aux) return TCS_OK;
        int st = cuda_status(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking), "cudaStreamCreate");
        for (int k = 0; k <= kBands && !st; k++)
            st = cuda_status(cudaEventCreateWithFlags(&band_ev[k], cudaEventDisableTiming), "cudaEventCreate");
        return st;
    }
    // band k: plane rows [q0, q1) and the grid rows [r0, r1) they hold
    void band(int k, int &q0, int &q1, int &r0, int &r1) const {
        const int nyp = g.p16.nyp;
        q0 = (int)((long long)nyp * k / kBands);
        q1 = (int)((long long)nyp * (k + 1) / kBands);
        r0 = std::max(0, q0 - kPadTop);
        r1 = std::min(prob.ny, q1 - kPadTop);
    }

    // Tile columns of the plain FP16 tensor sweeps (64, 96 or 128,
    // tcs_plan_set_tile_width); the other forms use 128.
    int tile_w = kTile;
    long long tiles() const {
        return (long long)((g.ny + kTile - 1) / kTile) * ((g.nx + tile_w - 1) / tile_w);
    }

    // t0: steps of the current run done before this one (split scale slots)
    int step(int from, cudaStream_t s, int t0 = 0) {
        return run_step(g, prob.stencil, prob.engine, prob.precision, coeffs, buf[from][0],
                        buf[from][1], buf[1 - from][0], buf[1 - from][1], s, tile_w, d_scale, t0);
    }

    // Temporal depth 2 (split precision on the tensor engine): steps run in
    // blocked pairs, with the same bits as single steps.
    int temporal_depth = 1;
    bool pairs() const { return temporal_depth == 2; }
    int step2(int from, cudaStream_t s, int t0) {
        return cuda_status(
            launch_tc_split2(g, prob.stencil, coeffs, static_cast<const uint16_t *>(buf[from][0]),
                             static_cast<const uint16_t *>(buf[from][1]),
                             static_cast<uint16_t *>(buf[1 - from][0]),
                             static_cast<uint16_t *>(buf[1 - from][1]), s, d_scale, t0),
            "blocked sweep launch");
    }
    // Tensor-engine plans (FP16 or split, temporal depth 1) run all steps of
    // a call in one launch, whose tiles of step j wait only for the
    // neighbouring tile rows of step j-1 (tcs_plan_set_multistep; TCS_MULTI=0
    // in the environment: one launch per step).  Measured on GB300 (FP16 box2d2r, us per step, one
    // launch per step -> one launch): 8196² 49.8 -> 42.2, 4096² 13.2 -> 10.4,
    // 2048² 6.8 -> 6.9, 1026² 5.5 -> 6.3: small grids are latency-bound, and
    // a step boundary between launches is quicker than the counters.
    int multistep = -1;
    bool multi() const {
        static const bool on = [] {
            const char *e = getenv("TCS_MULTI");
            return !(e && e[0] == '0');
        }();
        if (!on || !rows_done || prob.engine != TCS_ENGINE_TENSOR || pairs()) return false;
        if (multistep >= 0) return multistep == 1;
        const long long tiles = this->tiles();
        const long long sms = device_sms();
        // Split, us per step, one launch per step -> one launch (box2d1r /
        // box2d2r): 2400² 16.5 -> 11.8 / 16.5 -> 12.6, 3200² 22.2 -> 16.3 /
        // 23.0 -> 17.2, 4800² 51.8 -> 46.2 / 53.0 -> 47.0, 6400² 65.9 -> 60.5
        // / 66.4 -> 64.3, 8196² 104.0 -> 100.8 / 104.7 -> 107.2, 12000² 206.0
        // -> 208.9 / 207.5 -> 222.3, 16386² 378.6 -> 391.1 / 380.1 -> 416.9:
        // the multi-step kernel spends a little more per tile, which the step
        // overheads repay up to about 20 tiles per SM.
        if (prob.precision == TCS_PREC_SPLIT) return tiles > sms && tiles <= 20 * sms;
        return tiles > 2 * sms;
    }
    int steps_in_one(int steps, int from, cudaStream_t s) {
        const int tiles_y = (g.ny + kTile - 1) / kTile;
        int st = cuda_status(
            cudaMemsetAsync(rows_done, 0, (size_t)tiles_y * kRowCounterStride * sizeof(unsigned), s),
            "row counter reset");
        if (st) return st;
        const cudaError_t e =
            prob.precision == TCS_PREC_SPLIT
                ? launch_tc_split_steps(g, prob.stencil, coeffs, static_cast<const uint16_t *>(buf[from][0]),
                                        static_cast<const uint16_t *>(buf[from][1]),
                                        static_cast<uint16_t *>(buf[1 - from][0]),
                                        static_cast<uint16_t *>(buf[1 - from][1]), steps, rows_done, s,
                                        d_scale, 0)
                : launch_tc_f16_steps(g, prob.stencil, coeffs, static_cast<const uint16_t *>(buf[from][0]),
                                      static_cast<uint16_t *>(buf[1 - from][0]), steps, rows_done, s,
                                      tile_w);
        return cuda_status(e, "multi-step sweep launch");
    }
    // The state `steps` steps from `from` ends in: one flip per step.
    int final_state(int steps, int from) const {
        const int launches = pairs() ? steps / 2 + steps % 2 : steps;
        return from ^ (launches & 1);
    }
    // Enqueues `steps` steps from state `from` (one run); returns the final
    // state in *to.  A split run ends by moving its last two steps' scale
    // records into the places the next run starts from.
    int enqueue(int steps, int from, cudaStream_t s, int *to) {
        int st = TCS_OK;
        if (steps >= 2 && multi()) {
            *to = from ^ (steps & 1);
            st = steps_in_one(steps, from, s);
        } else {
            for (int t = 0; t < steps && !st;) {
                if (pairs() && steps - t >= 2) {
                    st = step2(from, s, t);
                    t += 2;
                } else {
                    st = step(from, s, t);
                    t += 1;
                }
                from ^= 1;
            }
            *to = from;
        }
        if (!st && d_scale)
            st = cuda_status(launch_split_scale_end_run(d_scale, steps, s), "scale end of run");
        return st;
    }
};

namespace {

int ensure_staging(tcs_plan p) {
    if (p->staging) return TCS_OK;
    return dev_alloc_t(&p->staging, (size_t)p->prob.ny * p->prob.nx * sizeof(float), "staging");
}

}  // namespace

extern "C" {

int tcs_plan_create(const tcs_problem *pr, tcs_plan *out) {
    if (!pr || !out || !pr->coeffs) return fail(TCS_ERR_INVALID, "tcs_plan_create: null argument");
    *out = nullptr;
    int st = check_mode(pr->engine, pr->precision);
    if (st) return st;
    std::unique_ptr<tcs_plan_s> p(new tcs_plan_s());
    p->prob = *pr;
    st = make_geom(pr->ny, pr->nx, pr->stencil, pr->y0, pr->y1, pr->x0, pr->x1, &p->g);
    if (st) return st;
    st = check_split_coeffs(pr->stencil, pr->precision, pr->coeffs);
    if (st) return st;
    const int n = 2 * stencil_r(pr->stencil) + 1;
    for (int k = 0; k < 25; k++) p->coeffs[k] = k < n * n ? pr->coeffs[k] : 0.0f;
    p->prob.coeffs = p->coeffs;
    const size_t elems = tcs_plane_elems(pr->ny, pr->nx, pr->precision);
    p->plane_bytes = elems * (pr->precision == TCS_PREC_F32 ? 4 : 2);
    // Zeroed, so that padding cells, which no sweep writes, are finite: a
    // zero band entry times a NaN would still poison an MMA sum.
    for (int s = 0; s < 2; s++)
        for (int pl = 0; pl < p->planes(); pl++) {
            st = dev_alloc_t(&p->buf[s][pl], p->plane_bytes, "plane");
            if (!st) st = cuda_status(cudaMemset(p->buf[s][pl], 0, p->plane_bytes), "cudaMemset(plane)");
            if (st) return st;
        }
    if (pr->precision == TCS_PREC_SPLIT) {
        st = dev_alloc_t(&p->d_scale, sizeof(SplitScale), "scale");
        if (!st) st = cuda_status(cudaMemset(p->d_scale, 0, sizeof(SplitScale)), "cudaMemset(scale)");
        if (st) return st;
    }
    if (pr->engine == TCS_ENGINE_TENSOR) {
        st = cuda_status(tc_prepare(pr->stencil, pr->precision == TCS_PREC_SPLIT), "tensor kernel set-up");
        if (st) return st;
        {
            const int tiles_y = (pr->ny + kTile - 1) / kTile;
            st = dev_alloc_t(&p->rows_done, (size_t)tiles_y * kRowCounterStride * sizeof(unsigned), "row counters");
            if (st) return st;
        }
    }
    *out = p.release();
    return TCS_OK;
}

int tcs_plan_destroy(tcs_plan plan) {
    delete plan;
    return TCS_OK;
}

int tcs_plan_set_coeffs(tcs_plan p, const float *coeffs) {
    if (!p || !coeffs) return fail(TCS_ERR_INVALID, "tcs_plan_set_coeffs: null argument");
    const int n = 2 * stencil_r(p->prob.stencil) + 1;
    int st = check_split_coeffs(p->prob.stencil, p->prob.precision, coeffs);
    if (st) return st;
    if (std::memcmp(p->coeffs, coeffs, n * n * sizeof(float)) != 0) {
        std::memcpy(p->coeffs, coeffs, n * n * sizeof(float));
        p->drop_graphs();  // graphs hold the coefficients as kernel parameters
    }
    return TCS_OK;
}

int tcs_plan_upload(tcs_plan p, const float *grid, int on_host, void *stream) {
    if (!p || !grid) return fail(TCS_ERR_INVALID, "tcs_plan_upload: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    const float *src = grid;
    if (on_host && p->banded()) {
        int st = ensure_staging(p);
        if (!st) st = p->ensure_bands();
        if (st) return st;
        p->cur = 0;
        const size_t row = (size_t)p->prob.nx;
        const bool f32 = p->prob.precision == TCS_PREC_F32;
        for (int k = 0; k < tcs_plan_s::kBands && !st; k++) {
            int q0, q1, r0, r1;
            p->band(k, q0, q1, r0, r1);
            if (r1 > r0)
                st = cuda_status(cudaMemcpyAsync(p->staging + r0 * row, grid + r0 * row,
                                                 (size_t)(r1 - r0) * row * sizeof(float),
                                                 cudaMemcpyHostToDevice, s), "upload copy");
            if (!st) st = cuda_status(cudaEventRecord(p->band_ev[k], s), "cudaEventRecord");
            if (!st) st = cuda_status(cudaStreamWaitEvent(p->aux, p->band_ev[k], 0), "cudaStreamWaitEvent");
            if (!st)
                st = cuda_status(launch_pack_rows(p->staging, p->prob.ny, p->prob.nx, f32,
                                                  p->buf[0][0], q0, q1, p->aux), "pack launch");
        }
        if (!st) st = cuda_status(cudaEventRecord(p->band_ev[tcs_plan_s::kBands], p->aux), "cudaEventRecord");
        if (!st) st = cuda_status(cudaStreamWaitEvent(s, p->band_ev[tcs_plan_s::kBands], 0), "cudaStreamWaitEvent");
        return st;
    }
    if (on_host) {
        int st = ensure_staging(p);
        if (st) return st;
        st = cuda_status(cudaMemcpyAsync(p->staging, grid, (size_t)p->prob.ny * p->prob.nx * sizeof(float),
                                         cudaMemcpyHostToDevice, s), "upload copy");
        if (st) return st;
        src = p->staging;
    }
    p->cur = 0;
    cudaError_t e;
    if (p->prob.precision == TCS_PREC_F32)
        e = launch_pack_f32(src, p->prob.ny, p->prob.nx, 0, 0.0f, static_cast<float *>(p->buf[0][0]), s);
    else if (p->prob.precision == TCS_PREC_SPLIT) {
        // scale so that max |x| 2^-E < 1, all on the device: the maximum, the
        // packing with its exponent, and the scale record's starting history
        int st = TCS_OK;
        if (!p->d_max) st = dev_alloc_t(&p->d_max, sizeof(unsigned), "max");
        if (!st) st = cuda_status(cudaMemsetAsync(p->d_max, 0, sizeof(unsigned), s), "memset(max)");
        if (!st) st = cuda_status(launch_max_abs(src, (size_t)p->prob.ny * p->prob.nx, p->d_max, s), "max_abs launch");
        if (!st)
            st = cuda_status(launch_pack_split_dev(src, p->prob.ny, p->prob.nx, p->d_max, nullptr,
                                                   static_cast<uint16_t *>(p->buf[0][0]),
                                                   static_cast<uint16_t *>(p->buf[0][1]), s),
                             "pack launch");
        if (st) return st;
        e = launch_split_scale_init(p->d_scale, p->d_max, p->g,
                                    static_cast<const uint16_t *>(p->buf[0][0]),
                                    static_cast<const uint16_t *>(p->buf[0][1]), s);
    }
    else
        e = launch_pack_f16(src, p->prob.ny, p->prob.nx, 0, 0.0f, static_cast<uint16_t *>(p->buf[0][0]), s);
    return cuda_status(e, "pack launch");
}

int tcs_plan_download(tcs_plan p, float *grid, int on_host, void *stream) {
    if (!p || !grid) return fail(TCS_ERR_INVALID, "tcs_plan_download: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (on_host && p->banded()) {
        int st = ensure_staging(p);
        if (!st) st = p->ensure_bands();
        if (st) return st;
        const size_t row = (size_t)p->prob.nx;
        const bool f32 = p->prob.precision == TCS_PREC_F32;
        st = cuda_status(cudaEventRecord(p->band_ev[tcs_plan_s::kBands], s), "cudaEventRecord");
        if (!st) st = cuda_status(cudaStreamWaitEvent(p->aux, p->band_ev[tcs_plan_s::kBands], 0), "cudaStreamWaitEvent");
        for (int k = 0; k < tcs_plan_s::kBands && !st; k++) {
            int q0, q1, r0, r1;
            p->band(k, q0, q1, r0, r1);
            st = cuda_status(launch_unpack_rows(p->buf[p->cur][0], p->prob.ny, p->prob.nx, f32,
                                                p->staging, q0, q1, p->aux), "unpack launch");
            if (!st) st = cuda_status(cudaEventRecord(p->band_ev[k], p->aux), "cudaEventRecord");
            if (!st) st = cuda_status(cudaStreamWaitEvent(s, p->band_ev[k], 0), "cudaStreamWaitEvent");
            if (!st && r1 > r0)
                st = cuda_status(cudaMemcpyAsync(grid + r0 * row, p->staging + r0 * row,
                                                 (size_t)(r1 - r0) * row * sizeof(float),
                                                 cudaMemcpyDeviceToHost, s), "download copy");
        }
        return st;
    }
    float *dst = grid;
    if (on_host) {
        int st = ensure_staging(p);
        if (st) return st;
        dst = p->staging;
    }
    cudaError_t e;
    const int c = p->cur;
    if (p->prob.precision == TCS_PREC_F32)
        e = launch_unpack_f32(static_cast<float *>(p->buf[c][0]), p->prob.ny, p->prob.nx, 0, dst, s);
    else if (p->prob.precision == TCS_PREC_SPLIT)
        e = launch_unpack_split_dev(static_cast<uint16_t *>(p->buf[c][0]), static_cast<uint16_t *>(p->buf[c][1]),
                                    p->prob.ny, p->prob.nx, split_scale_exp_ptr(p->d_scale), dst, s);
    else
        e = launch_unpack_f16(static_cast<uint16_t *>(p->buf[c][0]), p->prob.ny, p->prob.nx, 0, dst, s);
    int st = cuda_status(e, "unpack launch");
    if (st || !on_host) return st;
    return cuda_status(cudaMemcpyAsync(grid, p->staging, (size_t)p->prob.ny * p->prob.nx * sizeof(float),
                                       cudaMemcpyDeviceToHost, s), "download copy");
}

int tcs_plan_set_temporal_depth(tcs_plan p, int depth) {
    if (!p || depth < 1 || depth > 2) return fail(TCS_ERR_INVALID, "tcs_plan_set_temporal_depth: depth is 1 or 2");
    if (depth == 2 && !(p->prob.engine == TCS_ENGINE_TENSOR && p->prob.precision == TCS_PREC_SPLIT))
        return fail(TCS_ERR_UNSUPPORTED, "temporal depth 2 is built for split precision on the tensor engine");
    if (depth != p->temporal_depth) {
        p->temporal_depth = depth;
        p->drop_graphs();  // graphs hold the launch sequence
    }
    return TCS_OK;
}

int tcs_plan_set_multistep(tcs_plan p, int mode) {
    if (!p || mode < -1 || mode > 1) return fail(TCS_ERR_INVALID, "tcs_plan_set_multistep: mode is -1, 0 or 1");
    if (mode != p->multistep) {
        p->multistep = mode;
        p->drop_graphs();  // graphs hold the launch sequence
    }
    return TCS_OK;
}

int tcs_plan_set_tile_width(tcs_plan p, int tile_w) {
    if (!p || !valid_tile_width(tile_w))
        return fail(TCS_ERR_INVALID, "tcs_plan_set_tile_width: the width is 64, 96 or 128");
    if (tile_w != kTile &&
        !(p->prob.engine == TCS_ENGINE_TENSOR && p->prob.precision == TCS_PREC_F16))
        return fail(TCS_ERR_UNSUPPORTED, "tile widths below 128 are built for FP16 tensor sweeps");
    if (tile_w != p->tile_w) {
        p->tile_w = tile_w;
        p->drop_graphs();  // graphs hold the launch parameters
    }
    return TCS_OK;
}

int tcs_plan_tile_width(tcs_plan p, int *tile_w) {
    if (!p || !tile_w) return fail(TCS_ERR_INVALID, "tcs_plan_tile_width: null argument");
    *tile_w = p->tile_w;
    return TCS_OK;
}

int tcs_plan_launches(tcs_plan p, int steps, int *launches) {
    if (!p || steps < 0 || !launches) return fail(TCS_ERR_INVALID, "tcs_plan_launches: bad arguments");
    if (steps >= 2 && p->multi()) *launches = 1;
    else *launches = p->pairs() ? steps / 2 + steps % 2 : steps;
    return TCS_OK;
}

int tcs_plan_state(tcs_plan p, void **hi, void **lo, size_t *plane_bytes) {
    if (!p) return fail(TCS_ERR_INVALID, "tcs_plan_state: null plan");
    if (hi) *hi = p->buf[p->cur][0];
    if (lo) *lo = p->buf[p->cur][1];
    if (plane_bytes) *plane_bytes = p->plane_bytes;
    return TCS_OK;
}

int tcs_plan_scale_exp(tcs_plan p, int *scale_exp) {
    if (!p || !scale_exp) return fail(TCS_ERR_INVALID, "tcs_plan_scale_exp: null argument");
    *scale_exp = 0;
    if (!p->d_scale) return TCS_OK;
    return cuda_status(cudaMemcpy(scale_exp, split_scale_exp_ptr(p->d_scale), sizeof(int),
                                  cudaMemcpyDeviceToHost),
                       "scale exponent copy");
}

int tcs_plan_run(tcs_plan p, int steps, int use_graph, void *stream) {
    if (!p || steps < 0) return fail(TCS_ERR_INVALID, "tcs_plan_run: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (!use_graph || steps <= 1) {
        int to = p->cur;
        const int st = p->enqueue(steps, p->cur, s, &to);
        if (!st) p->cur = to;
        return st;
    }
    const auto key = std::make_pair(steps, p->cur);
    auto it = p->graphs.find(key);
    if (it == p->graphs.end()) {
        if (!p->capture_stream) {
            int st = cuda_status(cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking),
                                 "cudaStreamCreate");
            if (st) return st;
        }
        int st = cuda_status(cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal),
                             "cudaStreamBeginCapture");
        if (st) return st;
        int to = p->cur;
        const int launch_st = p->enqueue(steps, p->cur, p->capture_stream, &to);
        cudaGraph_t graph = nullptr;
        st = cuda_status(cudaStreamEndCapture(p->capture_stream, &graph), "cudaStreamEndCapture");
        if (launch_st || st) {
            if (graph) cudaGraphDestroy(graph);
            return launch_st ? launch_st : st;
        }
        cudaGraphExec_t exec = nullptr;
        st = cuda_status(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(graph);
        if (st) return st;
        it = p->graphs.emplace(key, exec).first;
    }
    int st = cuda_status(cudaGraphLaunch(it->second, s), "cudaGraphLaunch");
    if (st) return st;
    p->cur = p->final_state(steps, p->cur);
    return TCS_OK;
}

}  // extern "C"

// ======================================================== one-call form ==
namespace {

using CacheKey = std::tuple<int, int, int, int, int, int, int, int, int>;
struct PlanCache {
    std::map<CacheKey, tcs_plan> plans;
    ~PlanCache() {
        // Device memory is released by the driver at process exit; freeing it
        // from a static destructor could run after the CUDA runtime is gone.
        plans.clear();
    }
};
thread_local PlanCache t_cache;

}  // namespace

extern "C" {

int tcs_sweep_host(const float *h_in, float *h_out, const tcs_problem *pr, int steps) {
    if (!h_in || !h_out || !pr || !pr->coeffs || steps < 0)
        return fail(TCS_ERR_INVALID, "tcs_sweep_host: bad arguments");
    const CacheKey key{pr->ny, pr->nx, pr->stencil, pr->engine, pr->precision,
                       pr->y0, pr->y1, pr->x0, pr->x1};
    tcs_plan p;
    auto it = t_cache.plans.find(key);
    if (it == t_cache.plans.end()) {
        int st = tcs_plan_create(pr, &p);
        if (st) return st;
        t_cache.plans.emplace(key, p);
    } else {
        p = it->second;
    }
    int st = tcs_plan_set_coeffs(p, pr->coeffs);
    if (!st) st = tcs_plan_upload(p, h_in, 1, nullptr);
    if (!st) st = tcs_plan_run(p, steps, 1, nullptr);
    if (!st) st = tcs_plan_download(p, h_out, 1, nullptr);
    if (!st) st = cuda_status(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    if (!st) st = tcs_device_error(nullptr);
    return st;
}

void tcs_release_cache(void) {
    for (auto &kv : t_cache.plans) tcs_plan_destroy(kv.second);
    t_cache.plans.clear();
}

}  // extern "C"

// ================================================================= pipes ==
// Submission k runs on plan and stream k % 2; before a slot is reused its
// previous submission is waited for on the host.  Split plans keep their scale
// in device memory (maximum, exponent and packing on the stream), so no
// submission blocks the host, and results match tcs_sweep_host.
struct tcs_pipe_s {
    tcs_plan plan[2] = {nullptr, nullptr};
    cudaStream_t stream[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    cudaEvent_t swept[2] = {nullptr, nullptr};  // a slot's sweeps have finished
    long long submitted = 0;
    ~tcs_pipe_s() {
        for (int k = 0; k < 2; k++) {
            if (stream[k]) cudaStreamSynchronize(stream[k]);
            if (done[k]) cudaEventDestroy(done[k]);
            if (swept[k]) cudaEventDestroy(swept[k]);
            if (stream[k]) cudaStreamDestroy(stream[k]);
            if (plan[k]) tcs_plan_destroy(plan[k]);
        }
    }
};

extern "C" {

int tcs_pipe_create(const tcs_problem *pr, tcs_pipe *out) {
    if (!pr || !out) return fail(TCS_ERR_INVALID, "tcs_pipe_create: null argument");
    *out = nullptr;
    std::unique_ptr<tcs_pipe_s> q(new tcs_pipe_s());
    int st = TCS_OK;
    for (int k = 0; k < 2 && !st; k++) {
        st = tcs_plan_create(pr, &q->plan[k]);
        if (!st) st = cuda_status(cudaStreamCreateWithFlags(&q->stream[k], cudaStreamNonBlocking), "cudaStreamCreate");
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&q->done[k], cudaEventDisableTiming), "cudaEventCreate");
        if (!st) st = cuda_status(cudaEventCreateWithFlags(&q->swept[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    if (st) return st;
    *out = q.release();
    return TCS_OK;
}

int tcs_pipe_destroy(tcs_pipe q) {
    delete q;
    return TCS_OK;
}

int tcs_pipe_submit(tcs_pipe q, const float *h_in, float *h_out, int steps) {
    if (!q || !h_in || !h_out || steps < 0) return fail(TCS_ERR_INVALID, "tcs_pipe_submit: bad arguments");
    const int k = (int)(q->submitted & 1);
    cudaStream_t s = q->stream[k];
    int st = TCS_OK;
    if (q->submitted >= 2) st = cuda_status(cudaEventSynchronize(q->done[k]), "cudaEventSynchronize");
    if (!st) st = tcs_plan_upload(q->plan[k], h_in, 1, s);
    // Sweeps take turns: a slot's sweeps start after the previous
    // submission's, so that only copies (and the small pack and unpack
    // kernels) overlap them.  Two sets of persistent sweeps sharing the SMs
    // would each wait on CTAs of the other.
    if (!st && q->submitted >= 1)
        st = cuda_status(cudaStreamWaitEvent(s, q->swept[k ^ 1], 0), "cudaStreamWaitEvent");
    if (!st) st = tcs_plan_run(q->plan[k], steps, 1, s);
    if (!st) st = cuda_status(cudaEventRecord(q->swept[k], s), "cudaEventRecord");
    if (!st) st = tcs_plan_download(q->plan[k], h_out, 1, s);
    if (!st) st = cuda_status(cudaEventRecord(q->done[k], s), "cudaEventRecord");
    if (!st) q->submitted++;
    return st;
}

int tcs_pipe_wait(tcs_pipe q) {
    if (!q) return fail(TCS_ERR_INVALID, "tcs_pipe_wait: null pipe");
    for (int k = 0; k < 2; k++) {
        const int st = cuda_status(cudaStreamSynchronize(q->stream[k]), "cudaStreamSynchronize");
        if (st) return st;
    }
    return tcs_device_error(nullptr);
}

// ============================================================ drop-in ==
int tcs_host_code(float *h_A, float *h_B, float *h_C, int N, int n, int stencil, int engine,
                  int run_times, int skip_times, int step_times, int tile_size) {
    (void)tile_size;  // tiles are the engine's own
    if (!h_A || !h_B || !h_C) return fail(TCS_ERR_INVALID, "host_code: null array");
    if (stencil < TCS_STAR2D1R || stencil > TCS_BOX2D2R) return fail(TCS_ERR_INVALID, "unknown stencil %d", stencil);
    if (n != 2 * stencil_r(stencil) + 1) return fail(TCS_ERR_INVALID, "host_code: n = %d does not match the stencil", n);
    if (N <= 0 || N % 16) return fail(TCS_ERR_INVALID, "host_code: N = %d must be a positive multiple of 16", N);
    const int pad = 16, Np = N + 2 * pad;
    tcs_step_args a;
    a.ny = Np; a.nx = Np;
    a.stencil = stencil; a.engine = engine; a.precision = TCS_PREC_F16;
    a.y0 = pad; a.y1 = pad + N; a.x0 = pad; a.x1 = pad + N;
    a.coeffs = h_B;
    int st = check_mode(engine, TCS_PREC_F16);
    if (st) return st;
    GridGeom g;
    st = make_geom(Np, Np, stencil, a.y0, a.y1, a.x0, a.x1, &g);
    if (st) return st;

    const size_t cells = (size_t)N * N, plane = tcs_plane_elems(Np, Np, TCS_PREC_F16) * sizeof(uint16_t);
    float *d_f32 = nullptr;
    uint16_t *d_A = nullptr, *d_C = nullptr;
    cudaEvent_t start = nullptr, stop = nullptr;
    auto cleanup = [&]() {
        if (d_f32) dev_free(d_f32);
        if (d_A) dev_free(d_A);
        if (d_C) dev_free(d_C);
        if (start) cudaEventDestroy(start);
        if (stop) cudaEventDestroy(stop);
    };
    st = dev_alloc_t(&d_f32, cells * sizeof(float), "Failed to allocate device memory for A");
    if (!st) st = dev_alloc_t(&d_A, plane, "Failed to allocate device memory for A");
    if (!st) st = dev_alloc_t(&d_C, plane, "Failed to allocate device memory for C");
    if (!st) st = cuda_status(cudaMemset(d_C, 0, plane), "cudaMemset(C)");
    if (!st) st = cuda_status(cudaMemcpy(d_f32, h_A, cells * sizeof(float), cudaMemcpyHostToDevice), "H2D copy of A");
    // array_float2half + padding_2D(pad 16, value 1.0) + brick_layout_2D
    if (!st) st = cuda_status(launch_pack_f16(d_f32, N, N, pad, 1.0f, d_A, nullptr), "pack launch");
    if (!st && engine == TCS_ENGINE_TENSOR)
        st = cuda_status(tc_prepare(stencil, false), "tensor kernel set-up");
    if (!st) st = cuda_status(cudaEventCreate(&start), "cudaEventCreate");
    if (!st) st = cuda_status(cudaEventCreate(&stop), "cudaEventCreate");
    double sum = 0.0;
    for (int t = 0; t < run_times && !st; t++) {
        float elapsed = 0.0f;
        st = cuda_status(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        if (!st) st = cuda_status(cudaEventRecord(start, nullptr), "cudaEventRecord");
        if (!st) st = run_step(g, stencil, engine, TCS_PREC_F16, h_B, d_A, nullptr, d_C, nullptr, nullptr);
        if (!st) st = cuda_status(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        if (!st) st = cuda_status(cudaEventRecord(stop, nullptr), "cudaEventRecord");
        if (!st) st = cuda_status(cudaEventSynchronize(stop), "cudaEventSynchronize");
        if (!st) st = cuda_status(cudaEventElapsedTime(&elapsed, start, stop), "cudaEventElapsedTime");
        if (t >= skip_times) sum += elapsed;
    }
    if (!st) {
        printf("[Time] Time used: %f ms\n", sum / (run_times - skip_times) / step_times);
        fflush(stdout);  // the line is grepped from pipes (ncu wrappers, tests)
        st = tcs_device_error(nullptr);
    }
    // reverse_layout_2D + interior copy + array_half2float
    if (!st) st = cuda_status(launch_unpack_f16(run_times > 0 ? d_C : d_A, N, N, pad, d_f32, nullptr), "unpack launch");
    if (!st) st = cuda_status(cudaMemcpy(h_C, d_f32, cells * sizeof(float), cudaMemcpyDeviceToHost), "D2H copy of C");
    cleanup();
    return st;
}

static void host_or_exit(float *h_A, float *h_B, float *h_C, int N, int n, int stencil, int engine) {
    const int st = tcs_host_code(h_A, h_B, h_C, N, n, stencil, engine, 500, 400, 1, 1);
    if (st != TCS_OK) {
        // common/common.hpp:10-16: print and exit(-1)
        printf("CUDA error : %s, %s\n", "host_code", tcs_last_error());
        exit(-1);
    }
}

void host_star2d1r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_STAR2D1R, TCS_ENGINE_TENSOR); }
void host_star2d2r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_STAR2D2R, TCS_ENGINE_TENSOR); }
void host_box2d1r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_BOX2D1R, TCS_ENGINE_TENSOR); }
void host_box2d2r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_BOX2D2R, TCS_ENGINE_TENSOR); }
void host_cc_star2d1r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_STAR2D1R, TCS_ENGINE_CUDACORE); }
void host_cc_star2d2r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_STAR2D2R, TCS_ENGINE_CUDACORE); }
void host_cc_box2d1r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_BOX2D1R, TCS_ENGINE_CUDACORE); }
void host_cc_box2d2r(float *h_A, float *h_B, float *h_C, int N, int n) { host_or_exit(h_A, h_B, h_C, N, n, TCS_BOX2D2R, TCS_ENGINE_CUDACORE); }

}  // extern "C"
