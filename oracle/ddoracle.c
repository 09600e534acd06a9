/*
 * CPU oracle for the distance-driven projector -- TEST INFRASTRUCTURE.
 * See ddoracle.h.  The walk itself lives in ddoracle_body.h and is
 * instantiated here at FP32 (ddo_f_*) and FP64 (ddo_d_*).
 *
 * Build with -ffp-contract=off so that x86-64 and aarch64 builds round alike
 * (the reference's own x86 build never fuses multiply-adds).
 */
#include "ddoracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define DDO_MAX_THREADS 256

/* min(ceil(V / 128), cores): ParaDisCPU2d.cpp:338-340. */
int ddo_default_threads(int nv)
{
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    int t = (nv - 1) / 128 + 1;
    if (cores > 0 && t > cores) t = (int)cores;
    if (t > DDO_MAX_THREADS) t = DDO_MAX_THREADS;
    return t < 1 ? 1 : t;
}

/* Compare-and-swap float accumulation, as the reference does for its
 * multi-threaded backprojectors (ParaDisCPU2d.cpp:12-16). */
static void ddo_f_atomic_add(float *p, float v)
{
    uint32_t *u = (uint32_t *)p;
    uint32_t old = __atomic_load_n(u, __ATOMIC_RELAXED), nw;
    do {
        float f;
        memcpy(&f, &old, 4);
        f += v;
        memcpy(&nw, &f, 4);
    } while (!__atomic_compare_exchange_n(u, &old, nw, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
}

static void ddo_d_atomic_add(double *p, double v)
{
    uint64_t *u = (uint64_t *)p;
    uint64_t old = __atomic_load_n(u, __ATOMIC_RELAXED), nw;
    do {
        double f;
        memcpy(&f, &old, 8);
        f += v;
        memcpy(&nw, &f, 8);
    } while (!__atomic_compare_exchange_n(u, &old, nw, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
}

#define T float
#define FN(name) ddo_f_##name
#include "ddoracle_body.h"
#undef T
#undef FN

#define T double
#define FN(name) ddo_d_##name
#include "ddoracle_body.h"
#undef T
#undef FN
