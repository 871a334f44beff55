/*
 * CPU oracle for the 2-D Jacobi sweep hot path (star2d1r, star2d2r, box2d1r,
 * box2d2r).  TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it as the checker.  Nothing in the
 * tcstencil_gb300 product links, loads or calls this file.
 *
 * What is restated here, and from where (paths are inside buaa-hipo/TCStencil):
 *
 *   oracle_gold_step_f32   common/gold_star2d1r.cpp:4-14, gold_star2d2r.cpp:4-16,
 *                          gold_box2d1r.cpp:3-15, gold_box2d2r.cpp:3-15.
 *                          Same tap order, same non-fused float arithmetic
 *                          (build with -ffp-contract=off), generalised to a
 *                          ny x nx grid and an explicit update rectangle.
 *   oracle_pad_2d          layout16/host_star2d1r.cu:63-75   (padding_2D)
 *   oracle_brick_2d        layout16/host_star2d1r.cu:77-88   (brick_layout_2D)
 *   oracle_unbrick_2d      layout16/host_star2d1r.cu:90-101  (reverse_layout_2D)
 *   oracle_f32_to_f16 /    common/common.hpp:146-160         (array_float2half /
 *   oracle_f16_to_f32                                         array_half2float)
 *   oracle_init_coe_star   layout16/host_star2d1r.cu:33-61, host_star2d2r.cu:33-67
 *   oracle_init_coe_box    layout16/host_box2d1r.cu:29-46,  host_box2d2r.cu:29-50
 *   oracle_check_error_2d  common/common.hpp:38-92 (checkError2D /
 *                          checkRelativeError2D: results and reported cells,
 *                          without the printing)
 *
 * Arithmetic contracts of the GPU engine (used as tighter checks than gold):
 *   oracle_step_f16cc   FP16 storage, FP32 coefficients, fmaf chain in gold's
 *                       tap order, RNE to FP16  (CUDA-core FP16 kernel).
 *   oracle_step_f16tc   FP16 storage, FP16 coefficients, exact products summed
 *                       in double, RNE to FP16   (tensor-core FP16 kernel).
 *   oracle_step_split   fixed-point hi + lo*2^-11 FP16 pair storage,
 *                       coefficients in three FP16 pieces, four products,
 *                       sum in double (split tensor kernel); the run of
 *                       several steps, oracle_sweep_split, follows the
 *                       engine's per-step scale exponent.
 *   oracle_step_f64     the same stencil in double (error reference).
 *
 * Threaded CPU timing of gold (the CPU baseline of bench.py):
 *   oracle_gold_loop_step,  gold's own loop shape (per-tap store into the
 *   oracle_gold_bench_bands output cell for box stencils), one grid, threads
 *                           on row bands.
 *
 * The FP16 conversion below is the IEEE-754 binary16 round-to-nearest-even
 * rule, written from the format definition.  Steps of large grids run on row
 * bands over POSIX threads; each cell's arithmetic is the same either way.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

enum { ST_STAR2D1R = 0, ST_STAR2D2R = 1, ST_BOX2D1R = 2, ST_BOX2D2R = 3 };

#define MAX_TAPS 25

/* Tap list of a stencil in the order gold sums it.  Returns the tap count;
 * fills the radius r and the coefficient-matrix width n = 2r+1. */
static int taps_for(int stencil, int *r, int *n, int *tdy, int *tdx) {
    int k = 0;
    switch (stencil) {
    case ST_STAR2D1R: /* gold_star2d1r.cpp:10-12: up, centre, down, left, right */
        *r = 1;
        tdy[k] = -1; tdx[k++] = 0;
        tdy[k] = 0;  tdx[k++] = 0;
        tdy[k] = 1;  tdx[k++] = 0;
        tdy[k] = 0;  tdx[k++] = -1;
        tdy[k] = 0;  tdx[k++] = 1;
        break;
    case ST_STAR2D2R: /* gold_star2d2r.cpp:10-14: column top to bottom, then row */
        *r = 2;
        for (int d = -2; d <= 2; d++) { tdy[k] = d; tdx[k++] = 0; }
        tdy[k] = 0; tdx[k++] = -2;
        tdy[k] = 0; tdx[k++] = -1;
        tdy[k] = 0; tdx[k++] = 1;
        tdy[k] = 0; tdx[k++] = 2;
        break;
    case ST_BOX2D1R: /* gold_box2d1r.cpp:11-13: k = 0..8, (k/3-1, k%3-1) */
    case ST_BOX2D2R: /* gold_box2d2r.cpp:11-13: k = 0..24, (k/5-2, k%5-2) */
        *r = stencil == ST_BOX2D1R ? 1 : 2;
        for (int i = 0; i < (2 * *r + 1) * (2 * *r + 1); i++) {
            tdy[k] = i / (2 * *r + 1) - *r;
            tdx[k++] = i % (2 * *r + 1) - *r;
        }
        break;
    default:
        return -1;
    }
    *n = 2 * *r + 1;
    return k;
}

int oracle_stencil_radius(int stencil) {
    int r, n, dy[MAX_TAPS], dx[MAX_TAPS];
    return taps_for(stencil, &r, &n, dy, dx) < 0 ? -1 : r;
}

/* Copies the tap table out (for tests that check the GPU tap order). */
int oracle_stencil_taps(int stencil, int *tdy, int *tdx) {
    int r, n;
    return taps_for(stencil, &r, &n, tdy, tdx);
}

static int is_box(int stencil) { return stencil == ST_BOX2D1R || stencil == ST_BOX2D2R; }

/* ---------------------------------------------------------------- FP16 --- */

static uint16_t f64_to_f16(double v) {
    uint16_t sign = signbit(v) ? 0x8000u : 0u;
    double a = fabs(v);
    if (isnan(v)) return 0x7e00u;
    if (a >= 65520.0) return sign | 0x7c00u;
    if (a < 6.103515625e-05) { /* below 2^-14: subnormal, step 2^-24 */
        double m = nearbyint(a * 16777216.0);
        return sign | (uint16_t)m; /* m == 1024 is the smallest normal */
    }
    int e;
    frexp(a, &e); /* a in [2^(e-1), 2^e) */
    int E = e - 1;
    double m = nearbyint(ldexp(a, 10 - E)); /* in [1024, 2048] */
    if (m == 2048.0) { m = 1024.0; E += 1; }
    if (E > 15) return sign | 0x7c00u;
    return sign | (uint16_t)((E + 15) << 10) | (uint16_t)((int)m - 1024);
}

static double f16_to_f64(uint16_t h) {
    int s = h >> 15, e = (h >> 10) & 0x1f, m = h & 0x3ff;
    double v;
    if (e == 0) v = ldexp((double)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = ldexp((double)(m | 0x400), e - 25);
    return s ? -v : v;
}

uint16_t oracle_f16_from_f64(double v) { return f64_to_f16(v); }
double oracle_f64_from_f16(uint16_t h) { return f16_to_f64(h); }

void oracle_f32_to_f16(const float *in, uint16_t *out, long n) {
    for (long i = 0; i < n; i++) out[i] = f64_to_f16((double)in[i]);
}

void oracle_f16_to_f32(const uint16_t *in, float *out, long n) {
    for (long i = 0; i < n; i++) out[i] = (float)f16_to_f64(in[i]);
}

/* ------------------------------------------------------------- layouts --- */

/* padding_2D (layout16/host_star2d1r.cu:63-75): size^2 -> (size+2h)^2. */
void oracle_pad_2d(const uint16_t *in, uint16_t *out, int size, int halo, uint16_t value) {
    int p = size + 2 * halo;
    for (int i = 0; i < p; i++)
        for (int j = 0; j < p; j++) {
            int in_range = i >= halo && i < size + halo && j >= halo && j < size + halo;
            out[(long)i * p + j] = in_range ? in[(long)(i - halo) * size + (j - halo)] : value;
        }
}

/* brick_layout_2D (layout16/host_star2d1r.cu:77-88) generalised to ny x nx:
 * nby = ceil(ny/b), nbx = ceil(nx/b) bricks of b x b; cells past the grid are
 * `fill`.  For ny == nx == a multiple of b it is the reference transform. */
void oracle_brick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, int b, uint16_t fill) {
    int nby = (ny + b - 1) / b, nbx = (nx + b - 1) / b;
    for (int i = 0; i < nby; i++)
        for (int j = 0; j < nbx; j++)
            for (int x = 0; x < b; x++)
                for (int y = 0; y < b; y++) {
                    int gy = i * b + x, gx = j * b + y;
                    long o = ((long)i * nbx + j) * b * b + x * b + y;
                    out[o] = (gy < ny && gx < nx) ? in[(long)gy * nx + gx] : fill;
                }
}

/* reverse_layout_2D (layout16/host_star2d1r.cu:90-101), generalised likewise. */
void oracle_unbrick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, int b) {
    int nbx = (nx + b - 1) / b;
    for (int gy = 0; gy < ny; gy++)
        for (int gx = 0; gx < nx; gx++) {
            int i = gy / b, x = gy % b, j = gx / b, y = gx % b;
            out[(long)gy * nx + gx] = in[((long)i * nbx + j) * b * b + x * b + y];
        }
}

/* init_coe for the star stencils (layout16/host_star2d1r.cu:33-61 for n = 3,
 * layout16/host_star2d2r.cu:33-67 for n = 5): `a` is the 16x16 vertical band
 * (A operand), `b` the horizontal band with its centre zeroed (B operand),
 * both clipped at the brick edge.  B is n x n FP16, row-major. */
void oracle_init_coe_star(const uint16_t *B, int n, uint16_t *a, uint16_t *b) {
    int r = n / 2;
    memset(a, 0, 256 * sizeof(uint16_t));
    memset(b, 0, 256 * sizeof(uint16_t));
    uint16_t vert[5], hori[5];
    for (int i = 0; i < n; i++) {
        hori[i] = B[r * n + i];
        vert[i] = B[r + i * n];
    }
    hori[r] = 0;
    /* interior rows of the band: entry (row i+r, col i+j) of a, (row i+j,
     * col i+r) of b */
    for (int i = 0; i < 16 - 2 * r; i++)
        for (int j = 0; j < n; j++) {
            a[(i + r) * 16 + i + j] = vert[j];
            b[(i + j) * 16 + i + r] = hori[j];
        }
    /* clipped rows at the top/bottom (a) and left/right columns (b): the
     * n-d taps of an edge row d cells from the brick edge that stay inside */
    for (int d = 1; d <= r; d++)
        for (int t = 0; t < n - d; t++) {
            a[(r - d) * 16 + t] = vert[d + t];                        /* top    */
            a[(15 - r + d) * 16 + (16 - (n - d)) + t] = vert[t];      /* bottom */
            b[t * 16 + (r - d)] = hori[d + t];                        /* left   */
            b[((16 - (n - d)) + t) * 16 + (15 - r + d)] = hori[t];    /* right  */
        }
}

/* init_coe for the box stencils (layout16/host_box2d1r.cu:29-46 for n = 3,
 * layout16/host_box2d2r.cu:29-50 for n = 5): n horizontal 16x16 bands, band z
 * built from row z of B, clipped at the brick edge. */
void oracle_init_coe_box(const uint16_t *B, int n, uint16_t *coe) {
    int r = n / 2;
    memset(coe, 0, (size_t)256 * n * sizeof(uint16_t));
    for (int z = 0; z < n; z++) {
        uint16_t *c = coe + z * 256;
        for (int i = 0; i < 16 - 2 * r; i++)
            for (int j = 0; j < n; j++)
                c[(i + j) * 16 + i + r] = B[z * n + j];
        for (int d = 1; d <= r; d++)
            for (int t = 0; t < n - d; t++) {
                c[t * 16 + (r - d)] = B[z * n + d + t];
                c[((16 - (n - d)) + t) * 16 + (15 - r + d)] = B[z * n + t];
            }
    }
}

/* ------------------------------------------------------------- sweeps --- */
/* Every step below computes each output cell with the same scalar code; a
 * step of a large grid splits its rows into bands over POSIX threads
 * (ORACLE_THREADS, default: the online processors), which changes no result
 * bit.  FP16 inputs are widened through a table of all 65536 values, built
 * once from f16_to_f64. */

static double g_f16tab[65536];
static pthread_once_t g_f16tab_once = PTHREAD_ONCE_INIT;

static void f16tab_init(void) {
    for (int h = 0; h < 65536; h++) g_f16tab[h] = f16_to_f64((uint16_t)h);
}

static const double *f16tab(void) {
    pthread_once(&g_f16tab_once, f16tab_init);
    return g_f16tab;
}

static void rect_default(int ny, int nx, int r, int *y0, int *y1, int *x0, int *x1) {
    if (*y0 == 0 && *y1 == 0 && *x0 == 0 && *x1 == 0) {
        *y0 = r; *y1 = ny - r; *x0 = r; *x1 = nx - r;
    }
}

enum { K_GOLD32, K_F64, K_F16CC, K_F32, K_F16TC, K_SPLIT };

typedef struct {
    int kind, ny, nx, stencil, y0, y1, x0, x1, nt, r, n, box;
    int tdy[MAX_TAPS], tdx[MAX_TAPS];
    long off[MAX_TAPS];
    const void *A, *Al;
    void *C, *Cl;
    const float *Bf;
    const double *Bd;
    float cf[MAX_TAPS];
    double cd[MAX_TAPS], chi[MAX_TAPS], cfl[MAX_TAPS], clo[MAX_TAPS], c3[MAX_TAPS];
    int shift;        /* split: the step's values are multiplied by 2^shift */
    double *rowmax;   /* split: per row, the largest |x'| stored (or NULL) */
} step_ctx;

/* Fills the tap table and the coefficient forms of each kind.  Returns -1 for
 * an unknown stencil. */
static int ctx_init(step_ctx *c, int kind, int ny, int nx, int stencil, int y0, int y1, int x0,
                    int x1) {
    memset(c, 0, sizeof(*c));
    c->kind = kind; c->ny = ny; c->nx = nx; c->stencil = stencil;
    c->nt = taps_for(stencil, &c->r, &c->n, c->tdy, c->tdx);
    if (c->nt < 0) return -1;
    rect_default(ny, nx, c->r, &y0, &y1, &x0, &x1);
    c->y0 = y0; c->y1 = y1; c->x0 = x0; c->x1 = x1;
    c->box = is_box(stencil);
    for (int k = 0; k < c->nt; k++) c->off[k] = (long)c->tdy[k] * nx + c->tdx[k];
    return 0;
}

static int coef_index(const step_ctx *c, int k) {
    return (c->tdy[k] + c->r) * c->n + c->tdx[k] + c->r;
}

static void ctx_coeffs(step_ctx *c) {
    for (int k = 0; k < c->nt; k++) {
        int q = coef_index(c, k);
        if (c->kind == K_F64) { c->cd[k] = c->Bd[q]; continue; }
        double v = c->Bf[q];
        c->cf[k] = c->Bf[q];
        if (c->kind == K_F16TC) c->cd[k] = f16_to_f64(f64_to_f16(v));
        if (c->kind == K_SPLIT) {
            c->chi[k] = nearbyint(v * 2048.0) / 2048.0;
            c->cfl[k] = f16_to_f64(f64_to_f16(v));
            double rem = (v - c->chi[k]) * 2048.0;
            c->clo[k] = f16_to_f64(f64_to_f16(rem));
            c->c3[k] = f16_to_f64(f64_to_f16(rem - c->clo[k]));
        }
    }
}

static int inside(const step_ctx *c, int i, int j) {
    return i >= c->y0 && i < c->y1 && j >= c->x0 && j < c->x1;
}

/* Rows [i0, i1) of one step. */
static void step_rows(const step_ctx *c, int i0, int i1) {
    const double *H = f16tab();
    const int nx = c->nx, nt = c->nt;
    for (int i = i0; i < i1; i++) {
        int row_in = i >= c->y0 && i < c->y1;
        switch (c->kind) {
        case K_GOLD32: { /* gold: only the rectangle is written */
            if (!row_in) break;
            const float *A = (const float *)c->A;
            float *C = (float *)c->C;
            for (int j = c->x0; j < c->x1; j++) {
                const float *p = A + (long)i * nx + j;
                float s;
                int k0;
                if (c->box) { s = 0.0f; k0 = 0; }             /* C[i][j] = 0; C += ... */
                else { s = p[c->off[0]] * c->cf[0]; k0 = 1; } /* a*b + c*d + ...      */
                for (int k = k0; k < nt; k++) s = s + p[c->off[k]] * c->cf[k];
                C[(long)i * nx + j] = s;
            }
            break;
        }
        case K_F32: { /* gold plus the fixed-border copy */
            const float *A = (const float *)c->A;
            float *C = (float *)c->C;
            for (int j = 0; j < nx; j++) {
                long o = (long)i * nx + j;
                if (!inside(c, i, j)) { C[o] = A[o]; continue; }
                const float *p = A + o;
                float s;
                int k0;
                if (c->box) { s = 0.0f; k0 = 0; }
                else { s = p[c->off[0]] * c->cf[0]; k0 = 1; }
                for (int k = k0; k < nt; k++) s = s + p[c->off[k]] * c->cf[k];
                C[o] = s;
            }
            break;
        }
        case K_F64: { /* only the rectangle is written */
            if (!row_in) break;
            const double *A = (const double *)c->A;
            double *C = (double *)c->C;
            for (int j = c->x0; j < c->x1; j++) {
                long o = (long)i * nx + j;
                double s = 0.0;
                for (int k = 0; k < nt; k++) s += A[o + c->off[k]] * c->cd[k];
                C[o] = s;
            }
            break;
        }
        case K_F16CC: {
            const uint16_t *A = (const uint16_t *)c->A;
            uint16_t *C = (uint16_t *)c->C;
            for (int j = 0; j < nx; j++) {
                long o = (long)i * nx + j;
                if (!inside(c, i, j)) { C[o] = A[o]; continue; }
                float acc = 0.0f;
                for (int k = 0; k < nt; k++) acc = fmaf((float)H[A[o + c->off[k]]], c->cf[k], acc);
                C[o] = f64_to_f16((double)acc);
            }
            break;
        }
        case K_F16TC: {
            const uint16_t *A = (const uint16_t *)c->A;
            uint16_t *C = (uint16_t *)c->C;
            for (int j = 0; j < nx; j++) {
                long o = (long)i * nx + j;
                if (!inside(c, i, j)) { C[o] = A[o]; continue; }
                double s = 0.0;
                for (int k = 0; k < nt; k++) s += H[A[o + c->off[k]]] * c->cd[k];
                C[o] = f64_to_f16(s);
            }
            break;
        }
        case K_SPLIT: {
            const uint16_t *Ah = (const uint16_t *)c->A, *Al = (const uint16_t *)c->Al;
            uint16_t *Ch = (uint16_t *)c->C, *Cl = (uint16_t *)c->Cl;
            const double sc = ldexp(1.0, c->shift);
            double m = 0.0; /* units of 2^-11 */
            for (int j = 0; j < nx; j++) {
                long o = (long)i * nx + j;
                if (!inside(c, i, j)) {
                    uint16_t h = Ah[o], l = Al[o];
                    if (c->shift) { /* the pair scaled by 2^shift, split again exactly */
                        double a = H[h] * 2048.0 * sc, ai = trunc(a);
                        double bb = (a - ai) + H[l] * sc, rb = nearbyint(bb);
                        h = f64_to_f16((ai + rb) / 2048.0);
                        l = f64_to_f16(bb - rb);
                    }
                    Ch[o] = h;
                    Cl[o] = l;
                    continue;
                }
                double main = 0.0, corr = 0.0;
                for (int k = 0; k < nt; k++) {
                    long q = o + c->off[k];
                    double xh = H[Ah[q]], xl = H[Al[q]];
                    main += c->chi[k] * xh;
                    corr += c->cfl[k] * xl + c->clo[k] * xh + c->c3[k] * xh;
                }
                double v = (main + corr / 2048.0) * sc;
                uint16_t h = f64_to_f16(nearbyint(v * 2048.0) / 2048.0);
                Ch[o] = h;
                Cl[o] = f64_to_f16((v - H[h]) * 2048.0);
                m = fmax(m, fabs(v * 2048.0));
            }
            if (c->rowmax) c->rowmax[i] = m / 2048.0;
            break;
        }
        }
    }
}

static int oracle_threads(void) {
    const char *e = getenv("ORACLE_THREADS");
    long t = e ? atol(e) : sysconf(_SC_NPROCESSORS_ONLN);
    return t < 1 ? 1 : t > 64 ? 64 : (int)t;
}

typedef struct { const step_ctx *c; int i0, i1; } band_job;

static void *band_job_run(void *p) {
    band_job *b = (band_job *)p;
    step_rows(b->c, b->i0, b->i1);
    return NULL;
}

/* One step over all ny rows, on row bands when the grid is large. */
static void run_step(const step_ctx *c) {
    int T = oracle_threads();
    if ((long)c->ny * c->nx < (1L << 18) || T == 1 || c->ny < 2 * T) {
        step_rows(c, 0, c->ny);
        return;
    }
    pthread_t tid[64];
    band_job jobs[64];
    for (int t = 0; t < T; t++) {
        jobs[t].c = c;
        jobs[t].i0 = (int)((long)c->ny * t / T);
        jobs[t].i1 = (int)((long)c->ny * (t + 1) / T);
        if (pthread_create(&tid[t], NULL, band_job_run, &jobs[t])) {
            step_rows(c, jobs[t].i0, jobs[t].i1);
            tid[t] = 0;
        }
    }
    for (int t = 0; t < T; t++)
        if (tid[t]) pthread_join(tid[t], NULL);
}

/* One gold step in FP32 over the update rectangle [y0,y1) x [x0,x1) (all zero
 * = gold's interior [r, n-r)).  C outside the rectangle is not written. */
int oracle_gold_step_f32(const float *A, const float *B, float *C, int ny, int nx, int stencil,
                         int y0, int y1, int x0, int x1) {
    step_ctx c;
    if (ctx_init(&c, K_GOLD32, ny, nx, stencil, y0, y1, x0, x1)) return -1;
    c.A = A; c.C = C; c.Bf = B;
    ctx_coeffs(&c);
    run_step(&c);
    return 0;
}

/* The register-accumulator gold step on rows [row0, row1) only, in the
 * calling thread (for the threaded CPU harness below). */
static void gold_f32_rows(const float *A, const float *B, float *C, int ny, int nx, int stencil,
                          int row0, int row1) {
    step_ctx c;
    if (ctx_init(&c, K_GOLD32, ny, nx, stencil, 0, 0, 0, 0)) return;
    c.A = A; c.C = C; c.Bf = B;
    ctx_coeffs(&c);
    step_rows(&c, row0, row1);
}

int oracle_step_f64(const double *A, const double *B, double *C, int ny, int nx, int stencil,
                    int y0, int y1, int x0, int x1) {
    step_ctx c;
    if (ctx_init(&c, K_F64, ny, nx, stencil, y0, y1, x0, x1)) return -1;
    c.A = A; c.C = C; c.Bd = B;
    ctx_coeffs(&c);
    run_step(&c);
    return 0;
}

/* CUDA-core FP16 contract: FP16 in, FP32 coefficients, acc = fmaf chain in
 * gold's tap order starting from 0, RNE to FP16.  Cells outside the update
 * rectangle copy the input. */
int oracle_step_f16cc(const uint16_t *A, const float *B, uint16_t *C, int ny, int nx, int stencil,
                      int y0, int y1, int x0, int x1) {
    step_ctx c;
    if (ctx_init(&c, K_F16CC, ny, nx, stencil, y0, y1, x0, x1)) return -1;
    c.A = A; c.C = C; c.Bf = B;
    ctx_coeffs(&c);
    run_step(&c);
    return 0;
}

/* FP32-storage contract: gold's exact arithmetic, cells outside the rectangle
 * copy the input (this is gold plus the fixed-border copy of a ping-pong). */
int oracle_step_f32(const float *A, const float *B, float *C, int ny, int nx, int stencil,
                    int y0, int y1, int x0, int x1) {
    step_ctx c;
    if (ctx_init(&c, K_F32, ny, nx, stencil, y0, y1, x0, x1)) return -1;
    c.A = A; c.C = C; c.Bf = B;
    ctx_coeffs(&c);
    run_step(&c);
    return 0;
}

/* Tensor-core FP16 contract: FP16 in, coefficients rounded to FP16, exact
 * products, the sum taken in double, RNE to FP16. */
int oracle_step_f16tc(const uint16_t *A, const float *B, uint16_t *C, int ny, int nx, int stencil,
                      int y0, int y1, int x0, int x1) {
    step_ctx c;
    if (ctx_init(&c, K_F16TC, ny, nx, stencil, y0, y1, x0, x1)) return -1;
    c.A = A; c.C = C; c.Bf = B;
    ctx_coeffs(&c);
    run_step(&c);
    return 0;
}

#define SPLIT_SCALE 2048.0 /* lo is stored scaled by 2^11 */

/* Split storage of x (the engine's split planes): x' = x 2^-e,
 * hi = fp16(rint(x' 2^11) 2^-11) (fixed point), lo = fp16((x' - hi) 2^11). */
void oracle_split_f64(const double *x, uint16_t *hi, uint16_t *lo, long n, int e) {
    for (long i = 0; i < n; i++) {
        double xs = ldexp(x[i], -e);
        uint16_t h = f64_to_f16(nearbyint(xs * SPLIT_SCALE) / SPLIT_SCALE);
        hi[i] = h;
        lo[i] = f64_to_f16((xs - f16_to_f64(h)) * SPLIT_SCALE);
    }
}

void oracle_join_f64(const uint16_t *hi, const uint16_t *lo, double *x, long n, int e) {
    for (long i = 0; i < n; i++)
        x[i] = ldexp(f16_to_f64(hi[i]) + f16_to_f64(lo[i]) / SPLIT_SCALE, e);
}

/* Split-precision contract (planes as oracle_split_f64 stores them; the
 * stencil is linear, so the scale exponent does not enter a step).  An FP32
 * coefficient c is held as ch = rint(c 2^11) 2^-11 (fixed point) plus
 * rem = (c - ch) 2^11 in two FP16 pieces, cl = fp16(rem), c3 = fp16(rem - cl),
 * and cf = fp16(c).  Four products:
 *   v = sum ch*xh + 2^-11 sum (cf*xl + cl*xh + c3*xh)      (in double here)
 * then hi' = fp16(rint(v 2^11) 2^-11), lo' = fp16((v - hi') 2^11).  Every
 * ch*xh is a multiple of 2^-22, so the first sum is exact on the GPU too. */
int oracle_step_split(const uint16_t *Ah, const uint16_t *Al, const float *B, uint16_t *Ch,
                      uint16_t *Cl, int ny, int nx, int stencil, int y0, int y1, int x0, int x1) {
    step_ctx c;
    if (ctx_init(&c, K_SPLIT, ny, nx, stencil, y0, y1, x0, x1)) return -1;
    c.A = Ah; c.Al = Al; c.C = Ch; c.Cl = Cl; c.Bf = B;
    ctx_coeffs(&c);
    run_step(&c);
    return 0;
}

/* ------------------------------------------------- multi-step sweeps --- */
/* Ping-pong with a fixed border: both buffers start as the input, each step
 * writes the update rectangle of the other buffer.  `grid` is updated in
 * place with the result after `steps` steps. */

int oracle_sweep_f32(float *grid, const float *B, int ny, int nx, int stencil, int steps,
                     int y0, int y1, int x0, int x1) {
    long cells = (long)ny * nx;
    float *tmp = (float *)malloc(cells * sizeof(float));
    if (!tmp) return -2;
    memcpy(tmp, grid, cells * sizeof(float));
    float *cur = grid, *nxt = tmp;
    for (int t = 0; t < steps; t++) {
        if (oracle_gold_step_f32(cur, B, nxt, ny, nx, stencil, y0, y1, x0, x1)) { free(tmp); return -1; }
        float *s = cur; cur = nxt; nxt = s;
    }
    if (cur != grid) memcpy(grid, cur, cells * sizeof(float));
    free(tmp);
    return 0;
}

int oracle_sweep_f64(double *grid, const double *B, int ny, int nx, int stencil, int steps,
                     int y0, int y1, int x0, int x1) {
    long cells = (long)ny * nx;
    double *tmp = (double *)malloc(cells * sizeof(double));
    if (!tmp) return -2;
    memcpy(tmp, grid, cells * sizeof(double));
    double *cur = grid, *nxt = tmp;
    for (int t = 0; t < steps; t++) {
        if (oracle_step_f64(cur, B, nxt, ny, nx, stencil, y0, y1, x0, x1)) { free(tmp); return -1; }
        double *s = cur; cur = nxt; nxt = s;
    }
    if (cur != grid) memcpy(grid, cur, cells * sizeof(double));
    free(tmp);
    return 0;
}

typedef int (*step16_fn)(const uint16_t *, const float *, uint16_t *, int, int, int, int, int, int, int);

static int sweep16(step16_fn fn, uint16_t *grid, const float *B, int ny, int nx, int stencil,
                   int steps, int y0, int y1, int x0, int x1) {
    long cells = (long)ny * nx;
    uint16_t *tmp = (uint16_t *)malloc(cells * sizeof(uint16_t));
    if (!tmp) return -2;
    uint16_t *cur = grid, *nxt = tmp;
    for (int t = 0; t < steps; t++) {
        if (fn(cur, B, nxt, ny, nx, stencil, y0, y1, x0, x1)) { free(tmp); return -1; }
        uint16_t *s = cur; cur = nxt; nxt = s;
    }
    if (cur != grid) memcpy(grid, cur, cells * sizeof(uint16_t));
    free(tmp);
    return 0;
}

int oracle_sweep_f16cc(uint16_t *grid, const float *B, int ny, int nx, int stencil, int steps,
                       int y0, int y1, int x0, int x1) {
    return sweep16(oracle_step_f16cc, grid, B, ny, nx, stencil, steps, y0, y1, x0, x1);
}

int oracle_sweep_f16tc(uint16_t *grid, const float *B, int ny, int nx, int stencil, int steps,
                       int y0, int y1, int x0, int x1) {
    return sweep16(oracle_step_f16tc, grid, B, ny, nx, stencil, steps, y0, y1, x0, x1);
}

/* frexp exponent of a positive normal FP32 value (v 2^-e in [0.5, 1)) in
 * *e; 0 for zero, subnormal or non-finite v (the part is absent). */
static int f32_exp(float v, int *e) {
    if (!(v >= 1.17549435e-38f) || !isfinite(v)) return 0;
    frexpf(v, e);
    return 1;
}

/* e(M) of M = max(m, b 2^d), m and b as FP32 values: the larger of the
 * present parts' exponents, 0 for none or for a non-finite m (no change),
 * clamped to [-64, 64] (the engine's rule). */
static int split_exp_of(float m, float b, int d) {
    if (!isfinite(m)) return 0;
    int em = 0, eb = 0;
    const int hm = f32_exp(m, &em), hb = f32_exp(b, &eb);
    if (!hm && !hb) return 0;
    eb += d;
    int e = !hb ? em : !hm ? eb : (em > eb ? em : eb);
    return e < -64 ? -64 : e > 64 ? 64 : e;
}

/* A split sweep of one run with the engine's per-step scale, from planes as
 * uploaded: they start in units of 2^E (*exp_io, the packing exponent) and
 * end in units of 2^E_T (written back to *exp_io).  Step t's exponent is
 * E_t = E_{t-2} + e(M_{t-2}) (E_{-1} = E_0 = the input's, e(M_{-1}) =
 * e(M_0) = 0), M_t = max(m_t, B 2^(E_0 - E_t)) with m_t the largest |x'|
 * the step stores in its update rectangle and B the largest |x'| of the
 * input's cells outside it (|x'| 2^11 = |hi 2^11 + lo| rounded once to
 * FP32); the step's values are multiplied by 2^(E_{t-1} - E_t). */
int oracle_sweep_split(uint16_t *hi, uint16_t *lo, const float *B, int ny, int nx, int stencil,
                       int steps, int y0, int y1, int x0, int x1, int *exp_io) {
    long cells = (long)ny * nx;
    uint16_t *th = (uint16_t *)malloc(cells * sizeof(uint16_t));
    uint16_t *tl = (uint16_t *)malloc(cells * sizeof(uint16_t));
    double *rowmax = (double *)malloc((size_t)ny * sizeof(double));
    int *E = (int *)malloc((size_t)(steps + 2) * sizeof(int));
    int *eM = (int *)malloc((size_t)(steps + 2) * sizeof(int));
    if (!th || !tl || !rowmax || !E || !eM) {
        free(th); free(tl); free(rowmax); free(E); free(eM);
        return -2;
    }
    step_ctx c0;
    if (ctx_init(&c0, K_SPLIT, ny, nx, stencil, y0, y1, x0, x1)) {
        free(th); free(tl); free(rowmax); free(E); free(eM);
        return -1;
    }
    const double *H = f16tab();
    float bu = 0.0f; /* the border's largest |x'| 2^11 */
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++)
            if (!inside(&c0, i, j)) {
                long o = (long)i * nx + j;
                bu = fmaxf(bu, (float)fabs(H[hi[o]] * 2048.0 + H[lo[o]]));
            }
    const float bm = bu / 2048.0f;
    const int e_b = *exp_io;
    E[0] = E[1] = *exp_io; /* index t + 1 */
    eM[0] = eM[1] = 0;
    uint16_t *ch = hi, *cl = lo, *nh = th, *nl = tl;
    int rc = 0;
    for (int t = 1; t <= steps; t++) {
        int et = E[t - 1] + eM[t - 1];
        int k = E[t] - et;
        k = k < -64 ? -64 : k > 64 ? 64 : k;
        step_ctx c;
        if (ctx_init(&c, K_SPLIT, ny, nx, stencil, y0, y1, x0, x1)) { rc = -1; break; }
        c.A = ch; c.Al = cl; c.C = nh; c.Cl = nl; c.Bf = B;
        ctx_coeffs(&c);
        c.shift = k;
        c.rowmax = rowmax;
        run_step(&c);
        double M = 0.0;
        for (int i = 0; i < ny; i++) M = fmax(M, rowmax[i]);
        E[t + 1] = et;
        eM[t + 1] = split_exp_of((float)M, bm, e_b - et);
        uint16_t *s = ch; ch = nh; nh = s;
        s = cl; cl = nl; nl = s;
    }
    if (!rc) *exp_io = E[steps + 1];
    if (ch != hi) { memcpy(hi, ch, cells * 2); memcpy(lo, cl, cells * 2); }
    free(th); free(tl); free(rowmax); free(E); free(eM);
    return rc;
}

/* ------------------------------------------------------ error metrics --- */
/* checkError2D (relative = 0) and checkRelativeError2D (relative = 1) of
 * common/common.hpp:38-92, as the reference's nvcc build computes them, over
 * rows [y_lb, y_ub) and columns [x_lb, x_ub) of an N-wide grid:
 *   - each cell's error is the FLOAT difference output - reference, widened
 *     to double; checkError2D takes its magnitude, checkRelativeError2D
 *     divides it (sign kept) by the reference, or by min_number (MIN_NUMBER,
 *     1e-6) where |reference| (a float magnitude) is below it;
 *   - the squares are summed in row-major order; the result is
 *     sqrt(sum / cells);
 *   - a running maximum starts at `tolerance` (TOLERANCE, 0.01); every cell
 *     whose error exceeds it (signed, for the relative form) is reported by a
 *     "Values at index (j,k) differ" line and becomes the new maximum.
 * Instead of printing, the cells of those lines go to msg_j / msg_k (up to
 * msg_cap of them) and their count to *messages; *max_error, *max_j, *max_k
 * get the final maximum and its cell (the "[Test] Max ... Error" line, which
 * the reference prints only when that cell is not (0, 0)). */
double oracle_check_error_2d(int N, const float *output, const float *reference, int y_lb,
                             int y_ub, int x_lb, int x_ub, int relative, double tolerance,
                             double min_number, double *max_error, int *max_j, int *max_k,
                             int *messages, int *msg_j, int *msg_k, int msg_cap) {
    double error = 0.0, mx = tolerance;
    int mj = 0, mk = 0, nmsg = 0;
    for (int j = y_lb; j < y_ub; j++)
        for (int k = x_lb; k < x_ub; k++) {
            float o = output[(long)j * N + k], r = reference[(long)j * N + k];
            double e = (double)(o - r);
            if (relative)
                e = fabsf(r) < min_number ? e / min_number : e / (double)r;
            else
                e = e < 0.0 ? -e : e;
            error += e * e;
            if (e > mx) {
                if (nmsg < msg_cap) { msg_j[nmsg] = j; msg_k[nmsg] = k; }
                nmsg++;
                mx = e;
                mk = k;
                mj = j;
            }
        }
    *max_error = mx;
    *max_j = mj;
    *max_k = mk;
    *messages = nmsg;
    return sqrt(error / ((y_ub - y_lb) * (x_ub - x_lb)));
}

/* ------------------------------------------------ gold's own loop shape --- */
/* One gold step written the way common/gold_*.cpp writes it, for timing the
 * reference's CPU code as it runs (oracle_gold_step_f32 above is the same
 * arithmetic with a register accumulator and a tap table):
 *   box stencils (gold_box2d1r.cpp:8-14, gold_box2d2r.cpp:8-14): the output
 *     cell is zeroed and then accumulated in place, one tap at a time, with
 *     the tap's row and column taken as k / n and k % n.  C may alias A as far
 *     as the compiler knows, so every tap reloads and stores the cell;
 *   star stencils (gold_star2d1r.cpp:8-13, gold_star2d2r.cpp:8-15): one
 *     expression of products summed left to right.
 * Rows [row0, row1) of the interior [r, ny-r) x [r, nx-r) are written. */
static void gold_loop_rows(const float *A, const float *B, float *C, int ny, int nx, int stencil,
                           int row0, int row1) {
    (void)ny;
    if (stencil == ST_BOX2D1R || stencil == ST_BOX2D2R) {
        int n = stencil == ST_BOX2D1R ? 3 : 5, r = n / 2;
        for (int i = row0; i < row1; i++)
            for (int j = r; j < nx - r; j++) {
                float *c = C + (long)i * nx + j;
                *c = 0;
                for (int k = 0; k < n * n; k++)
                    *c += A[(long)(i - r + k / n) * nx + (j - r + k % n)] * B[(k / n) * n + k % n];
            }
    } else if (stencil == ST_STAR2D1R) {
        for (int i = row0; i < row1; i++)
            for (int j = 1; j < nx - 1; j++) {
                const float *a = A + (long)i * nx + j;
                C[(long)i * nx + j] = a[-nx] * B[1] + a[0] * B[4] + a[nx] * B[7] + a[-1] * B[3] +
                                      a[1] * B[5];
            }
    } else {
        for (int i = row0; i < row1; i++)
            for (int j = 2; j < nx - 2; j++) {
                const float *a = A + (long)i * nx + j;
                C[(long)i * nx + j] = a[-2 * nx] * B[2] + a[-nx] * B[7] + a[0] * B[12] +
                                      a[nx] * B[17] + a[2 * nx] * B[22] + a[-2] * B[10] +
                                      a[-1] * B[11] + a[1] * B[13] + a[2] * B[14];
            }
    }
}

/* One step in gold's loop shape over gold's whole interior. */
int oracle_gold_loop_step(const float *A, const float *B, float *C, int ny, int nx, int stencil) {
    int r = oracle_stencil_radius(stencil);
    if (r < 0) return -1;
    gold_loop_rows(A, B, C, ny, nx, stencil, r, ny - r);
    return 0;
}

/* ---------------------------------------------- CPU throughput harness --- */
/* One grid, `threads` POSIX threads on row bands of gold's interior, `steps`
 * ping-pong steps with a barrier between steps (both buffers start as the
 * input, so the border stays fixed).  loop_shape 1 runs gold's own loop shape
 * (gold_loop_rows), 0 the register-accumulator form (oracle_gold_step_f32).
 * Returns elapsed wall seconds of the steps (buffers are set up before the
 * clock starts), or < 0 on error.  If `out` is not NULL the final state is
 * copied there. */
typedef struct {
    float *a, *b;
    const float *B;
    int ny, nx, stencil, steps, row0, row1, loop_shape;
    pthread_barrier_t *bar;
} band_arg;

static void *band_worker(void *p) {
    band_arg *g = (band_arg *)p;
    float *cur = g->a, *nxt = g->b;
    for (int t = 0; t < g->steps; t++) {
        if (g->row1 > g->row0) {
            if (g->loop_shape)
                gold_loop_rows(cur, g->B, nxt, g->ny, g->nx, g->stencil, g->row0, g->row1);
            else
                gold_f32_rows(cur, g->B, nxt, g->ny, g->nx, g->stencil, g->row0, g->row1);
        }
        pthread_barrier_wait(g->bar);
        float *s = cur; cur = nxt; nxt = s;
    }
    return NULL;
}

double oracle_gold_bench_bands(const float *init, const float *B, int ny, int nx, int stencil,
                               int steps, int threads, int loop_shape, float *out) {
    int r = oracle_stencil_radius(stencil);
    if (r < 0 || threads < 1 || steps < 0 || ny <= 2 * r) return -1.0;
    long cells = (long)ny * nx;
    float *a = (float *)malloc(cells * sizeof(float));
    float *b = (float *)malloc(cells * sizeof(float));
    band_arg *args = (band_arg *)calloc(threads, sizeof(band_arg));
    pthread_t *tid = (pthread_t *)calloc(threads, sizeof(pthread_t));
    if (!a || !b || !args || !tid) { free(a); free(b); free(args); free(tid); return -2.0; }
    memcpy(a, init, cells * sizeof(float));
    memcpy(b, init, cells * sizeof(float));
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)threads);
    int rows = ny - 2 * r;
    for (int t = 0; t < threads; t++) {
        args[t].a = a; args[t].b = b; args[t].B = B;
        args[t].ny = ny; args[t].nx = nx; args[t].stencil = stencil; args[t].steps = steps;
        args[t].row0 = r + (int)((long)rows * t / threads);
        args[t].row1 = r + (int)((long)rows * (t + 1) / threads);
        args[t].loop_shape = loop_shape;
        args[t].bar = &bar;
    }
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < threads; t++) pthread_create(&tid[t], NULL, band_worker, &args[t]);
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    pthread_barrier_destroy(&bar);
    if (out) memcpy(out, steps % 2 ? b : a, cells * sizeof(float));
    free(a); free(b); free(args); free(tid);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
