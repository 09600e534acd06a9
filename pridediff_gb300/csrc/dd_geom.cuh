// Geometry of the distance-driven (DD) projector, shared by the CUDA kernels
// and by a host build used in tests.
//
// Everything in this header reproduces, operation by operation, the FP32 /
// FP64 mix of deeprecon's CPU projectors (deeprecon/cpu/dis2d/*.cpp), so that
// the boundary arrays the kernels integrate over are bit-identical to the ones
// deeprecon's walk visits.  Each rounding step is written with an explicit
// round-to-nearest intrinsic so that nvcc never fuses a multiply and an add
// (the reference's x86 build never does).
//
// The one structural fact the kernels rely on: deeprecon advances the pixel
// boundary of a walk by repeated FP32 addition (`Point1Proj += PixInterval`,
// FanFlatDisCPU2d.cpp:125), which drifts by up to ~1e-3 mm over a 512-pixel
// line.  Within one binade [2^e, 2^(e+1)) of the running value that addition
// advances by a constant (PixInterval rounded to the binade's ulp grid), so
// the drifted sequence is exactly piecewise arithmetic with one piece per
// binade (~20 per line).  build_pieces() computes the pieces in closed form;
// the kernels then evaluate any boundary, and the integral of the pixel
// function up to any position, in O(1) -- see DdPiece / DdLine.
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define DD_HD __host__ __device__ __forceinline__
#else
#define DD_HD static inline
#endif

// Explicitly rounded arithmetic (no contraction on either side).
#if defined(__CUDA_ARCH__)
#define FADD(a, b) __fadd_rn((a), (b))
#define FSUB(a, b) __fsub_rn((a), (b))
#define FMUL(a, b) __fmul_rn((a), (b))
#define FDIV(a, b) __fdiv_rn((a), (b))
#define DADD(a, b) __dadd_rn((a), (b))
#define DSUB(a, b) __dsub_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#define DDIV(a, b) __ddiv_rn((a), (b))
#define DSQRT(a) __dsqrt_rn(a)
#else
// host build: compiled with -ffp-contract=off
#define FADD(a, b) ((float)(a) + (float)(b))
#define FSUB(a, b) ((float)(a) - (float)(b))
#define FMUL(a, b) ((float)(a) * (float)(b))
#define FDIV(a, b) ((float)(a) / (float)(b))
#define DADD(a, b) ((double)(a) + (double)(b))
#define DSUB(a, b) ((double)(a) - (double)(b))
#define DMUL(a, b) ((double)(a) * (double)(b))
#define DDIV(a, b) ((double)(a) / (double)(b))
#define DSQRT(a) sqrt((double)(a))
#endif

// ---------------------------------------------------------------------------
// Constants of the piece model
// ---------------------------------------------------------------------------
#define DD_EMIN (-6)          // |x| < 2^-6 mm shares the centre slot
#define DD_EMAX 16            // |x| >= 2^17 mm shares the outermost slots
#define DD_NEXP (DD_EMAX - DD_EMIN + 1)
#define DD_NSLOT (2 * DD_NEXP + 1)   // 47 value slots, monotone in the value
#define DD_SLOT_BYTES 48
#define DD_NPMAX 32           // pieces per line (a 512-pixel line needs ~21)

// Line-record flags
#define DD_LINE_SATURATED 1   // more binades than DD_NPMAX: tail approximated

// One arithmetic run of drifted boundaries: boundary index `gb` has value Q,
// index gb - n has value Q - n*dl (exact FP32 arithmetic inside a binade).
struct DdPiece {
    float Q;      // value of the run's last boundary
    float dl;     // constant increment of the run
    float invdl;  // 1 / dl
    int gb;       // absolute index of the run's last boundary
};

// Header of the record of one walked line (row or column) of one view.
// Boundary index i is the UPPER boundary of pixel i; the walk starts at
// `bound0` (lower boundary of pixel i0, lower boundary of bin idet0).
struct DdLineHdr {
    float bound0;   // start of the walk on the projection axis
    int i0;         // first walked pixel
    int nend;       // number of pixels on the line (last boundary = nend-1)
    int npiece;     // pieces in use (0: the line meets no detector bin)
    float endv;     // value of the last boundary (end of the walk)
    float alpha;    // per-line scale of the DD backprojector (VirDetSize/PixInterval)
    int idet0;      // first walked detector bin
    int flags;
};

// A full line record (592 bytes, 16-byte multiple so TMA can move it).
struct DdLine {
    DdLineHdr h;                      // 32 B
    unsigned char slot[DD_SLOT_BYTES];// value slot -> first piece whose Q >= slot start
    DdPiece p[DD_NPMAX];              // 512 B
};

// Per-view scalars (2-D).
struct DdView2 {
    int xb;        // 1: project on x, walk image rows; 0: on y, walk columns
    int flip;      // detector index reversed
    float s, c;    // FP32 sin / cos of the view angle
    float srcx, srcy;
    float det0, di;   // parallel beam: first detector boundary, pitch
    float det0xy;     // fan-flat: x (y) of virtual-detector boundary 0
    float axis0, axis1;   // image extent on the walked axis
    float pad;
};

// ---------------------------------------------------------------------------
// Float bit helpers
// ---------------------------------------------------------------------------
DD_HD int dd_fbits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_int(x);
#else
    union { float f; int i; } u; u.f = x; return u.i;
#endif
}
DD_HD float dd_bitsf(int i) {
#if defined(__CUDA_ARCH__)
    return __int_as_float(i);
#else
    union { float f; int i; } u; u.i = i; return u.f;
#endif
}
// Unbiased exponent of a normal float (|x| in [2^e, 2^(e+1))).
DD_HD int dd_fexp(float x) { return ((dd_fbits(x) >> 23) & 0xFF) - 127; }
// Binade identity of a value: sign and exponent (0 and subnormals: own id).
DD_HD int dd_binade(float x) {
    const int b = dd_fbits(x);
    const int e = (b >> 23) & 0xFF;
    if (e == 0) return 0;
    return (b < 0) ? -e : e;
}
// Value slot used to look pieces up (monotone non-decreasing in x).
DD_HD int dd_slot(float x) {
    const int b = dd_fbits(x);
    int e = ((b >> 23) & 0xFF) - 127;
    if (e < DD_EMIN) return DD_NEXP;
    if (e > DD_EMAX) e = DD_EMAX;
    const int k = e - DD_EMIN + 1;
    return (b < 0) ? DD_NEXP - k : DD_NEXP + k;
}
// Signed integer mantissa of a normal float on its binade's ulp grid.
DD_HD int dd_mant(float x) {
    const int b = dd_fbits(x);
    const int m = (b & 0x7FFFFF) | 0x800000;
    return (b < 0) ? -m : m;
}
// Float with signed mantissa m (|m| < 2^24) on the grid of exponent e.
DD_HD float dd_from_mant(int m, int e) {
    if (m == 0) return 0.0f;
    return ldexpf((float)m, e - 23);
}

// ---------------------------------------------------------------------------
// Piece builder: the drifted sequence b_{i+1} = fl(b_i + pint) for
// i = i0 .. nend-1, starting from b_{i0} = v0.  Returns the number of pieces.
// ---------------------------------------------------------------------------
DD_HD int dd_build_pieces(float v0, float pint, int i0, int nend, DdPiece *P, int *flags) {
    int np = 0;
    float x = v0;
    int i = i0;
    const int last = nend - 1;
    while (i <= last) {
        if (np == DD_NPMAX - 1) {
            // out of pieces: close the line with one approximate run
            P[np].Q = FADD(x, FMUL((float)(last - i), pint));
            P[np].dl = pint;
            P[np].invdl = 1.0f / pint;
            P[np].gb = last;
            np++;
            *flags |= DD_LINE_SATURATED;
            break;
        }
        const int bid = dd_binade(x);
        if (i == last) {
            P[np].Q = x; P[np].dl = pint; P[np].invdl = 1.0f / pint; P[np].gb = i; np++;
            break;
        }
        const float x1 = FADD(x, pint);
        if (dd_binade(x1) != bid || bid == 0) {
            const float d = FSUB(x1, x);
            P[np].Q = x; P[np].dl = d; P[np].invdl = 1.0f / d; P[np].gb = i; np++;
            x = x1; i += 1;
            continue;
        }
        if (i + 1 == last) {
            const float d = FSUB(x1, x);
            P[np].Q = x1; P[np].dl = d; P[np].invdl = 1.0f / d; P[np].gb = i + 1; np++;
            break;
        }
        const float x2 = FADD(x1, pint);
        if (dd_binade(x2) != bid) {
            const float d = FSUB(x1, x);
            P[np].Q = x1; P[np].dl = d; P[np].invdl = 1.0f / d; P[np].gb = i + 1; np++;
            x = x2; i += 2;
            continue;
        }
        // constant increment from x1 on (round-to-even ties settle after one step)
        const int e = dd_fexp(x1);
        const int M1 = dd_mant(x1);
        const int Dm = dd_mant(x2) - M1;          // increment in ulps (> 0)
        long long k;
        if (M1 > 0) k = ((long long)(1 << 24) - 1 - M1) / Dm;   // stay below 2^(e+1)
        else k = ((long long)(-(1 << 23)) - M1) / Dm;            // stay at or below -2^e
        if (k > (long long)(last - (i + 1))) k = last - (i + 1);
        const int MQ = M1 + (int)k * Dm;
        const float Q = dd_from_mant(MQ, e);
        const float d = FSUB(x2, x1);
        P[np].Q = Q; P[np].dl = d; P[np].invdl = 1.0f / d; P[np].gb = i + 1 + (int)k; np++;
        x = FADD(Q, pint);
        i = i + 2 + (int)k;
    }
    return np;
}

// slot map: slot -> first piece whose last value Q >= the slot's lowest value
DD_HD void dd_build_slots(const DdPiece *P, int np, unsigned char *slot) {
    int p = 0;
    for (int s = 0; s < DD_SLOT_BYTES; s++) {
        // the first piece whose slot is >= s
        while (p < np - 1 && dd_slot(P[p].Q) < s) p++;
        slot[s] = (unsigned char)p;
    }
}

// Piece that covers value d (d already clamped to [bound0, endv]).
DD_HD int dd_piece_of_value(const DdLine *L, float d) {
    int p = L->slot[dd_slot(d)];
    const int np = L->h.npiece;
    while (p < np - 1 && d > L->p[p].Q) p++;
    return p;
}

// Piece holding boundary index i (i in [i0, nend-1]); `hint` from the slot of
// an estimate of the value.
DD_HD int dd_piece_of_index(const DdLine *L, int i, float estimate) {
    int p = L->slot[dd_slot(estimate)];
    const int np = L->h.npiece;
    while (p < np - 1 && i > L->p[p].gb) p++;
    while (p > 0 && i <= L->p[p - 1].gb) p--;
    return p;
}

// Drifted value of boundary index i.
DD_HD float dd_boundary(const DdLine *L, int i, float estimate) {
    const int p = dd_piece_of_index(L, i, estimate);
    const DdPiece P = L->p[p];
    return FADD(P.Q, FMUL((float)(i - P.gb), P.dl));
}

// Locate value d: pixel j (whose lower boundary is index j-1) and the offset r
// of d past that lower boundary.  j is clamped to [i0, nend].
DD_HD void dd_locate(const DdLine *L, float d, int *pp, int *jj, float *rr) {
    const int p = dd_piece_of_value(L, d);
    const DdPiece P = L->p[p];
    const int n = (int)floorf(FMUL(FSUB(d, P.Q), P.invdl));
    int j = P.gb + n + 1;
    if (j < L->h.i0) j = L->h.i0;
    if (j > L->h.nend) j = L->h.nend;
    const float bv = FADD(P.Q, FMUL((float)(j - 1 - P.gb), P.dl));
    *pp = p;
    *jj = j;
    *rr = FSUB(d, bv);
}

// ---------------------------------------------------------------------------
// Reference-exact FP32 helpers (FanFlatDisCPU2d.cpp:11-26, FanArcDisCPU2d.cpp:11-29)
// ---------------------------------------------------------------------------
DD_HD float dd_map2x(float sx, float sy, float px, float py) {
    return FDIV(FSUB(FMUL(sx, py), FMUL(sy, px)), FSUB(py, sy));
}
DD_HD float dd_map2y(float sx, float sy, float px, float py) {
    return FDIV(FSUB(FMUL(sy, px), FMUL(sx, py)), FSUB(px, sx));
}
DD_HD float dd_tricos2(float a, float b) {
    const float q = FADD(FMUL(a, a), FMUL(b, b));
    return (float)DDIV(fabs((double)b), DSQRT((double)q));
}
DD_HD float dd_cw_flat(float sx, float sy, float px, float py, float r) {
    const float d = FDIV(FADD(FMUL(sx, px), FMUL(sy, py)), r);
    const float t = FSUB(r, d);
    return FDIV(FMUL(r, r), FMUL(t, t));
}
DD_HD float dd_cw_arc(float sx, float sy, float px, float py) {
    const float a = FSUB(sx, px), b = FSUB(sy, py);
    return FADD(FMUL(a, a), FMUL(b, b));
}
// floor() of a float expression evaluated as the reference does (the FP32
// quotient is promoted to double before flooring).
DD_HD int dd_ifloor(float q) {
#if defined(__CUDA_ARCH__)
    return (int)floorf(q);   // same value as the double floor for every float
#else
    return (int)floor((double)q);
#endif
}
