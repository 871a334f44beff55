/*
 * Per-variant `host_code` for the reference's unchanged drivers.
 *
 * The reference links exactly one host file per binary and calls
 *   extern "C" void host_code(float *h_A, float *h_B, float *h_C, int N, int n)
 * from common/main_1r.cu:28 / common/main_2r.cu:31 (prototype at
 * common/main_1r.cu:7).  This file is compiled once per (engine, stencil) with
 * -DTCS_STENCIL=<enum tcs_stencil> -DTCS_ENGINE=<enum tcs_engine> into a small
 * library exporting that symbol; the common/param.hpp macros RUN_TIMES,
 * SKIP_TIMES, STEP_TIMES and TILE_SIZE may be given with -D as the reference's
 * script/nvcc_compile.py does, and default to param.hpp's values.
 */
#include <stdio.h>
#include <stdlib.h>

#include "../../include/tcs.h"

#ifndef TCS_STENCIL
#error "define TCS_STENCIL"
#endif
#ifndef TCS_ENGINE
#error "define TCS_ENGINE"
#endif
#ifndef RUN_TIMES
#define RUN_TIMES 500
#endif
#ifndef STEP_TIMES
#define STEP_TIMES 1
#endif
#ifndef SKIP_TIMES
#define SKIP_TIMES 400
#endif
#ifndef TILE_SIZE
#define TILE_SIZE 1
#endif

void host_code(float *h_A, float *h_B, float *h_C, int N, int n) {
    int st = tcs_host_code(h_A, h_B, h_C, N, n, TCS_STENCIL, TCS_ENGINE, RUN_TIMES, SKIP_TIMES,
                           STEP_TIMES, TILE_SIZE);
    if (st != TCS_OK) {
        /* common/common.hpp:10-16: print the error and exit(-1) */
        printf("CUDA error : %s, %s\n", "host_code", tcs_last_error());
        exit(-1);
    }
}
