// FP64 drift check (tcs_drift_*): an FP64 shadow of a stencil problem on
// the device, stepped beside an FP16 or split sweep, and a reduction that
// measures how far an FP32 grid has drifted from it.  FP64 appears only here
// and in the oracle, never in the sweep kernels.
//
// The shadow steps with gold's tap order and separately rounded multiply and
// add (no fused multiply-add), the arithmetic of the FP64 restatement of
// common/gold_*.cpp in the oracle, so the two agree bit for bit.
#include <cstring>
#include <memory>

#include "tcs_internal.h"

namespace tcs {
namespace {

struct F64Taps {
    double c[25];  // in gold's tap order
    int dy[25], dx[25];
    int n;
};

__global__ void f64_step_kernel(const double *__restrict__ in, double *__restrict__ out, int ny,
                                int nx, int y0, int y1, int x0, int x1, const F64Taps t) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nx) return;
    for (int y = blockIdx.y; y < ny; y += gridDim.y) {
        const size_t o = (size_t)y * nx + x;
        if (y < y0 || y >= y1 || x < x0 || x >= x1) {
            out[o] = in[o];
            continue;
        }
        double s = 0.0;
        for (int k = 0; k < t.n; k++)
            s = __dadd_rn(s, __dmul_rn(in[(size_t)(y + t.dy[k]) * nx + x + t.dx[k]], t.c[k]));
        out[o] = s;
    }
}

__global__ void f32_to_f64_kernel(const float *__restrict__ in, double *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// acc[0] += sum (a - ref)^2, acc[1] += sum ref^2, acc[2] = max |a - ref|
__global__ void drift_reduce_kernel(const float *__restrict__ a, const double *__restrict__ ref,
                                    size_t n, double *acc) {
    double d2 = 0.0, r2 = 0.0, mx = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const double d = (double)a[i] - ref[i];
        d2 += d * d;
        r2 += ref[i] * ref[i];
        mx = fmax(mx, fabs(d));
    }
    for (int o = 16; o > 0; o >>= 1) {
        d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], d2);
        atomicAdd(&acc[1], r2);
        // non-negative doubles order like their bit patterns
        atomicMax(reinterpret_cast<unsigned long long *>(&acc[2]),
                  (unsigned long long)__double_as_longlong(mx));
    }
}

}  // namespace
}  // namespace tcs

using namespace tcs;

struct tcs_drift_s {
    GridGeom g;
    int stencil = 0;
    F64Taps taps;
    double *buf[2] = {nullptr, nullptr};
    int cur = 0;
    double *d_acc = nullptr;
    float *staging = nullptr;
    ~tcs_drift_s() {
        for (void *p : {(void *)buf[0], (void *)buf[1], (void *)d_acc, (void *)staging})
            if (p) dev_free(p);
    }
};

extern "C" {

int tcs_drift_create(const tcs_problem *pr, tcs_drift *out) {
    if (!pr || !out || !pr->coeffs) return fail(TCS_ERR_INVALID, "tcs_drift_create: null argument");
    *out = nullptr;
    std::unique_ptr<tcs_drift_s> d(new tcs_drift_s());
    int st = make_geom(pr->ny, pr->nx, pr->stencil, pr->y0, pr->y1, pr->x0, pr->x1, &d->g);
    if (st) return st;
    d->stencil = pr->stencil;
    const int r = stencil_r(pr->stencil), n = 2 * r + 1;
    d->taps.n = tap_count(pr->stencil);
    for (int k = 0; k < d->taps.n; k++) {
        d->taps.dy[k] = tap_dy(pr->stencil, k);
        d->taps.dx[k] = tap_dx(pr->stencil, k);
        d->taps.c[k] = (double)pr->coeffs[(d->taps.dy[k] + r) * n + d->taps.dx[k] + r];
    }
    const size_t bytes = (size_t)pr->ny * pr->nx * sizeof(double);
    for (int s = 0; s < 2 && !st; s++) st = dev_alloc_t(&d->buf[s], bytes, "drift");
    if (!st) st = dev_alloc_t(&d->d_acc, 3 * sizeof(double), "drift acc");
    if (st) return st;
    *out = d.release();
    return TCS_OK;
}

int tcs_drift_destroy(tcs_drift d) {
    delete d;
    return TCS_OK;
}

int tcs_drift_upload(tcs_drift d, const float *grid, int grid_on_host, void *stream) {
    if (!d || !grid) return fail(TCS_ERR_INVALID, "tcs_drift_upload: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)d->g.ny * d->g.nx;
    const float *src = grid;
    int st = TCS_OK;
    if (grid_on_host) {
        if (!d->staging) st = dev_alloc_t(&d->staging, n * sizeof(float), "drift staging");
        if (!st) st = cuda_status(cudaMemcpyAsync(d->staging, grid, n * sizeof(float), cudaMemcpyHostToDevice, s), "drift upload");
        if (st) return st;
        src = d->staging;
    }
    d->cur = 0;
    const unsigned blocks = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    f32_to_f64_kernel<<<blocks, 256, 0, s>>>(src, d->buf[0], n);
    return cuda_status(cudaGetLastError(), "drift upload kernel");
}

int tcs_drift_run(tcs_drift d, int steps, void *stream) {
    if (!d || steps < 0) return fail(TCS_ERR_INVALID, "tcs_drift_run: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 grid((d->g.nx + 127) / 128, d->g.ny < 65535 ? d->g.ny : 65535);
    for (int t = 0; t < steps; t++) {
        f64_step_kernel<<<grid, 128, 0, s>>>(d->buf[d->cur], d->buf[d->cur ^ 1], d->g.ny, d->g.nx,
                                             d->g.y0, d->g.y1, d->g.x0, d->g.x1, d->taps);
        int st = cuda_status(cudaGetLastError(), "drift step");
        if (st) return st;
        d->cur ^= 1;
    }
    return TCS_OK;
}

int tcs_drift_compare(tcs_drift d, const float *d_grid, double *rel_l2, double *max_abs,
                      void *stream) {
    if (!d || !d_grid) return fail(TCS_ERR_INVALID, "tcs_drift_compare: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)d->g.ny * d->g.nx;
    int st = cuda_status(cudaMemsetAsync(d->d_acc, 0, 3 * sizeof(double), s), "drift reset");
    if (st) return st;
    const unsigned blocks = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    drift_reduce_kernel<<<blocks, 256, 0, s>>>(d_grid, d->buf[d->cur], n, d->d_acc);
    double acc[3];
    st = cuda_status(cudaGetLastError(), "drift reduce");
    if (!st) st = cuda_status(cudaMemcpyAsync(acc, d->d_acc, sizeof(acc), cudaMemcpyDeviceToHost, s), "drift result");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (st) return st;
    if (rel_l2) *rel_l2 = acc[1] > 0 ? sqrt(acc[0] / acc[1]) : sqrt(acc[0]);
    if (max_abs) *max_abs = acc[2];
    return TCS_OK;
}

int tcs_drift_download(tcs_drift d, double *h_grid, void *stream) {
    if (!d || !h_grid) return fail(TCS_ERR_INVALID, "tcs_drift_download: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    int st = cuda_status(cudaMemcpyAsync(h_grid, d->buf[d->cur], (size_t)d->g.ny * d->g.nx * sizeof(double),
                                         cudaMemcpyDeviceToHost, s), "drift download");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return st;
}

int tcs_drift_state(tcs_drift d, const double **d_grid) {
    if (!d || !d_grid) return fail(TCS_ERR_INVALID, "tcs_drift_state: null argument");
    *d_grid = d->buf[d->cur];
    return TCS_OK;
}

}  // extern "C"
