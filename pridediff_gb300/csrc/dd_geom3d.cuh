// 3-D view, column, row and line set-up for cone-flat, cone-arc and spiral
// DD projection, plus the exact segment and z-walk weights shared by the
// forward-type and adjoint-type kernels (and by a host build used in tests).
//
// deeprecon has no CPU path for these geometries (RadonTorch.cpp:604); the
// arithmetic follows its CUDA kernels (ConeFlatDisCUDA3d.cu, ConeArcDisCUDA3d.cu,
// SpiralDisCUDA3d.cu), whose per-thread loop walks, for one (view, detector
// row) and one block of 256 detector columns, the merged sequence of drifted
// pixel boundaries and column boundaries of every image line, with an inner
// walk over the 1-3 slices that a (column, row) cell meets on that line.
//
// Here the merged walk is restated as a set of (pixel, column) overlap
// segments: segment (j, k) spans [max(PL_j, CL_k), min(PH_j, CH_k)], where the
// pixel interval [PL_j, PH_j] and the column interval [CL_k, CH_k] are the
// values the walk visits (the walk start replaces the first lower boundary
// of each sequence).  A forward-type kernel enumerates the segments of one
// column, an adjoint-type kernel those of one pixel; both compute the width
// as the same FP32 difference of the same two floats, so the pair is an
// exact transpose.  The drifted pixel boundaries come from the piece model
// of dd_geom.cuh, one record per (view, line, 256-column block) because the
// reference restarts the FP32 accumulation in every block.
#pragma once

#include "dd_geom.cuh"
#include "../../include/pridediff_dd.h"

enum { DD_GEOM3_CONE_FLAT = 0, DD_GEOM3_CONE_ARC = 1, DD_GEOM3_SPIRAL = 2 };
#define DD3_CHUNK 256   // detector columns per walk block (ConeFlatDisCUDA3d.cu:53-56)

// Per-view scalars (3-D).  128 bytes.
struct DdView3 {
    int xb;          // 1: project on x, walk image rows; 0: on y, walk columns
    int flip;        // detector column index reversed
    float flag;      // -1 when flipped, else 1
    float s, c;      // FP32 sin / cos of the (spiral-corrected) source angle
    float view;      // angles[v]
    float srcx, srcy, srcz;
    float colsz;     // column pitch (arc / spiral: radians, spiral-corrected)
    float colshift;  // column shift (arc / spiral: radians, spiral-corrected)
    float sdd, iso;  // source-detector / source-isocentre distance (spiral-corrected)
    float axial;     // spiral: table position of the view
    float vds, vbs;  // cone-flat: virtual column pitch / shift
    float di;        // cone-flat: column pitch projected on the axis
    float bp_scale;  // per-bin scale of the DD backprojector family
    float axis0, axis1;   // image extent on the walked axis
    float z0, z1;         // volume extent in z
    float magmin, magmax; // range of the per-column row magnification
    float rzA, rzB;       // row0z(r) ~= rzA + r * rzB (row candidate search)
    float pad[6];
};
// the view record and the line record are moved by bulk copies: sizes must be
// multiples of 16 bytes (and arrays of them keep every element 16-byte aligned)
static_assert(sizeof(DdView3) == 128, "DdView3 must be 128 bytes");
static_assert(sizeof(DdLine) % 16 == 0, "DdLine must be a multiple of 16 bytes");

// Per-(view, line) z quantities: p0z, p1z (volume z extent on the line's
// plane), pintz (slice pitch there), parea (pixel area for the DD-BP family).
// Stored as float4 {p0z, p1z, pintz, parea}.

// Approximate quotient for estimates that are corrected afterwards.
DD_HD float dd3_approx_div(float num, float den) {
#if defined(__CUDA_ARCH__)
    return __fdividef(num, den);
#else
    return num / den;
#endif
}

// deeprecon's 3-D kernels evaluate sin, cos and tan of FP32 angles and atan of
// an FP32 ratio with the device's single-precision functions
// (ConeFlatDisCUDA3d.cu:62-63, ConeArcDisCUDA3d.cu:9-14, :69-70, :118-119,
// SpiralDisCUDA3d.cu:76-77), and the compiler fuses the arc boundary
// sourcex + sourcey * tan(a) into one multiply-add.  The device build calls
// the same functions and the same fused operation, so that view and column
// geometry round as the reference's do: the arc boundaries land within a few
// ulps of the correctly rounded values, which is up to 1e-4 of a 0.3 mm cell.
// The host build (the CPU model tests) rounds the double functions.
DD_HD float dd3_sin(float a) {
#if defined(__CUDA_ARCH__)
    return sinf(a);
#else
    return (float)sin((double)a);
#endif
}
DD_HD float dd3_cos(float a) {
#if defined(__CUDA_ARCH__)
    return cosf(a);
#else
    return (float)cos((double)a);
#endif
}
DD_HD float dd3_tan(float a) {
#if defined(__CUDA_ARCH__)
    return tanf(a);
#else
    return (float)tan((double)a);
#endif
}
DD_HD float dd3_atan(float a) {
#if defined(__CUDA_ARCH__)
    return atanf(a);
#else
    return (float)atan((double)a);
#endif
}
DD_HD float dd3_mul_add(float a, float b, float c) {   // a * b + c
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return a * b + c;
#endif
}

// ---------------------------------------------------------------------------
// View set-up: ConeFlatDisCUDA3d.cu:62-105, ConeArcDisCUDA3d.cu:40-60,
// SpiralDisCUDA3d.cu:39-82.  sp4 = {axial, radius shift, angle shift, axial
// shift} of the view (spiral only).
// ---------------------------------------------------------------------------
DD_HD void dd3_view_scalars(int geom, const dd_geom3d *g, float view, const float *sp4, DdView3 *w) {
    const float R = g->iso_source, SDD = g->source_detector;
    float dc = g->col_size, cshift = g->col_shift;
    float ang = view;
    w->view = view;
    w->iso = R;
    w->sdd = SDD;
    w->srcz = 0.0f;
    w->axial = 0.0f;
    w->vds = w->vbs = w->di = 0.0f;
    if (geom == DD_GEOM3_SPIRAL) {
        const float axial = sp4[0], drad = sp4[1], dang = sp4[2], daxial = sp4[3];
        w->iso = FADD(R, drad);
        w->sdd = FADD(SDD, drad);
        dc = FDIV(FMUL(g->col_size, SDD), w->sdd);
        cshift = FSUB(FDIV(FMUL(g->col_shift, SDD), w->sdd), FDIV(FMUL(dang, FSUB(w->sdd, w->iso)), w->sdd));
        ang = FADD(view, dang);
        w->srcz = FADD(axial, daxial);
        w->axial = axial;
    }
    w->colsz = dc;
    w->colshift = cshift;
    const float s = dd3_sin(ang), c = dd3_cos(ang);
    w->s = s;
    w->c = c;
    w->xb = FMUL(c, c) > 0.5f;
    w->flip = w->xb ? (c < 0.0f) : (s < 0.0f);
    w->flag = w->flip ? -1.0f : 1.0f;
    w->srcx = FMUL(-s, w->iso);
    w->srcy = FMUL(c, w->iso);
    if (geom == DD_GEOM3_CONE_FLAT) {
        w->vds = FMUL(FDIV(R, SDD), dc);
        w->vbs = FMUL(FDIV(R, SDD), cshift);
        w->di = FMUL(w->vds, fabsf(w->xb ? c : s));
        w->bp_scale = w->vds;
    } else {
        w->bp_scale = FMUL(w->iso, dc);
    }
    const int W = g->width, H = g->height, Dp = g->depth;
    if (w->xb) {
        w->axis0 = (float)DADD(DMUL(-W / 2.0, (double)g->pix_x), (double)g->pix_xshift);
        w->axis1 = (float)DADD(DMUL(W / 2.0, (double)g->pix_x), (double)g->pix_xshift);
    } else {
        w->axis0 = (float)DADD(DMUL(-H / 2.0, (double)g->pix_y), (double)g->pix_yshift);
        w->axis1 = (float)DADD(DMUL(H / 2.0, (double)g->pix_y), (double)g->pix_yshift);
    }
    const double pzs = (geom == DD_GEOM3_SPIRAL) ? 0.0 : (double)g->pix_zshift;
    w->z0 = (float)DADD(DMUL(-Dp / 2.0, (double)g->pix_z), pzs);
    w->z1 = (float)DADD(DMUL(Dp / 2.0, (double)g->pix_z), pzs);
    w->magmin = w->magmax = 1.0f;
    w->rzA = w->rzB = 0.0f;
    for (int i = 0; i < 6; i++) w->pad[i] = 0.0f;
}

// Sorted column boundary k (0..C) on the projection axis.
DD_HD float dd3_col_boundary(int geom, const dd_geom3d *g, const DdView3 *w, int k) {
    const int C = g->num_col;
    if (geom == DD_GEOM3_CONE_FLAT) {
        const double u = w->flip ? DADD(DMUL(DSUB(C / 2.0, (double)k), (double)w->vds), (double)w->vbs)
                                 : DADD(DMUL(DSUB((double)k, C / 2.0), (double)w->vds), (double)w->vbs);
        const float dx = (float)DMUL(u, (double)w->c), dy = (float)DMUL(u, (double)w->s);
        return w->xb ? dd_map2x(w->srcx, w->srcy, dx, dy) : dd_map2y(w->srcx, w->srcy, dx, dy);
    }
    // ConeArcDisCUDA3d.cu:49-55 (uses the view angle without the spiral shift)
    const double a = w->flip
        ? DADD(DADD(DMUL(DSUB(C / 2.0, (double)k), (double)w->colsz), (double)w->colshift), (double)w->view)
        : DADD(DADD(DMUL(DSUB((double)k, C / 2.0), (double)w->colsz), (double)w->colshift), (double)w->view);
    const float t = dd3_tan((float)a);
    return w->xb ? dd3_mul_add(w->srcy, t, w->srcx) : FADD(w->srcy, FDIV(w->srcx, t));
}

// Row magnification of sorted column k onto the line plane
// (ConeFlatDisCUDA3d.cu:70-76, ConeArcDisCUDA3d.cu:51-58).
DD_HD float dd3_col_mag(int geom, const dd_geom3d *g, const DdView3 *w, int k) {
    const int C = g->num_col;
    float cen;
    if (geom == DD_GEOM3_CONE_FLAT) {
        const double u = w->flip
            ? DADD(DMUL(DSUB(DSUB(C / 2.0, (double)k), 0.5), (double)w->vds), (double)w->vbs)
            : DADD(DMUL(DSUB(DADD((double)k, 0.5), C / 2.0), (double)w->vds), (double)w->vbs);
        cen = w->xb ? (float)DMUL(u, (double)w->s) : (float)DMUL(u, (double)w->c);
    } else {
        const float a1 = w->flip
            ? (float)DADD(DADD(DMUL(DSUB(DSUB(C / 2.0, (double)k), 1.0), (double)w->colsz), (double)w->colshift), (double)w->view)
            : (float)DADD(DADD(DMUL(DSUB((double)(k + 1), C / 2.0), (double)w->colsz), (double)w->colshift), (double)w->view);
        const double ac = w->flip ? DADD((double)a1, DMUL(0.5, (double)w->colsz))
                                  : DSUB((double)a1, DMUL(0.5, (double)w->colsz));
        cen = w->xb ? (float)DADD(DMUL(-cos(ac), (double)w->sdd), (double)w->srcy)
                    : (float)DADD(DMUL(sin(ac), (double)w->sdd), (double)w->srcx);
    }
    return w->xb ? FDIV(w->srcy, FSUB(w->srcy, cen)) : FDIV(w->srcx, FSUB(w->srcx, cen));
}

// Lower / upper z of detector row r before the per-column magnification
// (ConeFlatDisCUDA3d.cu:68-69, ConeArcDisCUDA3d.cu:40-41, SpiralDisCUDA3d.cu:49).
DD_HD void dd3_row_z(int geom, const dd_geom3d *g, const DdView3 *w, int r, float *z0, float *z1) {
    const int Rn = g->num_row;
    const double rr = DSUB((double)r, Rn / 2.0);
    if (geom == DD_GEOM3_CONE_FLAT) {
        const float R = g->iso_source, SDD = g->source_detector;
        *z0 = (float)DDIV(DMUL(DADD(DMUL(rr, (double)g->row_size), (double)g->row_shift), (double)R), (double)SDD);
        *z1 = FADD(*z0, FMUL(FDIV(R, SDD), g->row_size));
    } else if (geom == DD_GEOM3_CONE_ARC) {
        *z0 = (float)DADD(DMUL(rr, (double)g->row_size), (double)g->row_shift);
        *z1 = FADD(*z0, g->row_size);
    } else {
        *z0 = (float)DADD(DADD(DMUL(rr, (double)g->row_size), (double)w->axial), (double)g->row_shift);
        *z1 = FADD(*z0, g->row_size);
    }
}

// Row boundaries of row (z0, z1) under column magnification `mag` on the
// line plane.
DD_HD void dd3_rp(int geom, const DdView3 *w, float mag, float z0, float z1, float *rp0, float *rp1) {
    if (geom == DD_GEOM3_SPIRAL) {
        *rp0 = FADD(FMUL(mag, FSUB(z0, w->srcz)), w->srcz);
        *rp1 = FADD(FMUL(mag, FSUB(z1, w->srcz)), w->srcz);
    } else {
        *rp0 = FMUL(mag, z0);
        *rp1 = FMUL(mag, z1);
    }
}

// Per-bin scale of Proj / ProjTrans for sorted column [d0, d1] and row
// [rp0, rp1] (ConeFlatDisCUDA3d.cu:77-84).
DD_HD float dd3_proj_scale(const dd_geom3d *g, const DdView3 *w, float d0, float d1, float rp0, float rp1) {
    const float coef1 = FMUL(FSUB(d1, d0), FSUB(rp1, rp0));
    const float a = (float)DSUB(DDIV((double)FADD(d1, d0), 2.0), (double)(w->xb ? w->srcx : w->srcy));
    const float b = (float)DDIV((double)FADD(rp1, rp0), 2.0);
    const float cc = w->xb ? w->srcy : w->srcx;
    const float q = FADD(FADD(FMUL(a, a), FMUL(b, b)), FMUL(cc, cc));
    const float coef2 = FDIV(fabsf(cc), (float)DSQRT((double)q));
    return FDIV(w->xb ? g->pix_y : g->pix_x, FMUL(coef1, coef2));
}

// Centre of walked line `line` (row y for x-branch views, column x otherwise).
DD_HD float dd3_line_pos(const dd_geom3d *g, const DdView3 *w, int line) {
    const int W = g->width, H = g->height;
    return w->xb
        ? (float)DADD(DMUL(DSUB(DSUB(H / 2.0, (double)line), 0.5), (double)g->pix_y), (double)g->pix_yshift)
        : (float)DADD(DMUL(DADD(DSUB((double)line, W / 2.0), 0.5), (double)g->pix_x), (double)g->pix_xshift);
}

// Line magnification onto its plane.
DD_HD float dd3_line_mag(const DdView3 *w, float lpos) {
    return w->xb ? FDIV(w->srcy, FSUB(w->srcy, lpos)) : FDIV(w->srcx, FSUB(w->srcx, lpos));
}

// Pixel centre of pixel j on a line (the FBP weight is evaluated there).  The
// reference evaluates (j + 0.5) * pitch + axis0 in FP64 and rounds to FP32;
// one FMA of the exact j + 0.5 rounds the exact value once, the same float
// unless it lies within 2^-53 (relative) of an FP32 rounding boundary, at the
// FP32 rate (this runs once per segment and view).
DD_HD void dd3_pix_centre(const dd_geom3d *g, const DdView3 *w, float lpos, int j, float *px, float *py) {
    if (w->xb) {
        *px = fmaf((float)j + 0.5f, g->pix_x, w->axis0);
        *py = lpos;
    } else {
        *px = lpos;
        *py = fmaf((float)j + 0.5f, g->pix_y, w->axis0);
    }
}

// Per-line set-up for walk block cc (columns cc*256 ...): the walk start and
// the drifted pixel boundaries (ConeFlatDisCUDA3d.cu:106-130,
// ConeArcDisCUDA3d.cu:84-96, SpiralDisCUDA3d.cu:93-105).  lz receives
// {p0z, p1z, pintz, parea}; L->h.alpha holds parea as well.
DD_HD void dd3_line_setup(int geom, const dd_geom3d *g, const DdView3 *w, const float *dp, int line, int cc,
                          float *lz, DdLine *L) {
    const int W = g->width, H = g->height, Dp = g->depth, C = g->num_col;
    const int xb = w->xb;
    const int npix = xb ? W : H;
    const float lpos = dd3_line_pos(g, w, line);
    float p0, p1;
    if (xb) {
        p0 = dd_map2x(w->srcx, w->srcy, w->axis0, lpos);
        p1 = dd_map2x(w->srcx, w->srcy, w->axis1, lpos);
    } else {
        p0 = dd_map2y(w->srcx, w->srcy, lpos, w->axis0);
        p1 = dd_map2y(w->srcx, w->srcy, lpos, w->axis1);
    }
    const float m = dd3_line_mag(w, lpos);
    float p0z, p1z;
    if (geom == DD_GEOM3_SPIRAL) {
        p0z = FADD(FMUL(m, FSUB(w->z0, w->srcz)), w->srcz);
        p1z = FADD(FMUL(m, FSUB(w->z1, w->srcz)), w->srcz);
    } else {
        p0z = FMUL(m, w->z0);
        p1z = FMUL(m, w->z1);
    }
    const float pint = FDIV(FSUB(p1, p0), (float)npix);
    const float pintz = FDIV(FSUB(p1z, p0z), (float)Dp);
    const float parea = FMUL(pint, pintz);
    lz[0] = p0z;
    lz[1] = p1z;
    lz[2] = pintz;
    lz[3] = parea;

    const int c0 = cc * DD3_CHUNK;
    const int maxn = (C - c0 < DD3_CHUNK) ? C - c0 : DD3_CHUNK;
    int ipix, idet;
    float bound0;
    if (geom == DD_GEOM3_CONE_FLAT) {
        bound0 = p0 > dp[c0] ? p0 : dp[c0];
        if (p0 == bound0) {
            const float back = xb
                ? FDIV(FMUL(w->srcy, bound0), FADD(FDIV(FMUL(FSUB(bound0, w->srcx), w->s), w->c), w->srcy))
                : FDIV(FMUL(w->srcx, bound0), FADD(FDIV(FMUL(FSUB(bound0, w->srcy), w->c), w->s), w->srcx));
            const double uc = w->flip ? DADD(DMUL(DSUB(C / 2.0, (double)c0), (double)w->vds), (double)w->vbs)
                                      : DADD(DMUL(DSUB((double)c0, C / 2.0), (double)w->vds), (double)w->vbs);
            const float col0 = xb ? (float)DMUL(uc, (double)w->c) : (float)DMUL(uc, (double)w->s);
            ipix = 0;
            idet = dd_ifloor(FDIV(FSUB(back, col0), w->di));
        } else {
            ipix = dd_ifloor(FDIV(FSUB(bound0, p0), pint));
            idet = 0;
        }
    } else {
        const float base = FADD(w->colshift, w->view);
        float tan0, tan1;
        if (xb) {
            const float dxs = FSUB(w->srcx, p0);
            tan0 = (dxs == 0.0f) ? 1e10f : FDIV(w->srcy, dxs);
            tan1 = (base == 0.0f) ? 1e10f : FDIV(-1.0f, dd3_tan(base));
        } else {
            tan0 = FDIV(FSUB(w->srcy, p0), w->srcx);
            tan1 = FDIV(-1.0f, dd3_tan(base));
        }
        const float q = FDIV(FSUB(tan0, tan1), FADD(1.0f, FMUL(tan0, tan1)));
        const float delta = dd3_atan(q);
        const double kd = DADD(DSUB(C / 2.0, (double)c0), (double)FDIV(FMUL(delta, w->flag), w->colsz));
        idet = (int)floor(kd);
        if (idet < 0) {
            bound0 = dp[c0];
            ipix = dd_ifloor(FDIV(FSUB(bound0, p0), pint));
            idet = 0;
        } else {
            bound0 = p0;
            ipix = 0;
        }
    }
    if (idet < 0) idet = 0;
    if (ipix < 0) ipix = 0;   // the reference would read outside the volume there
    DdLineHdr &h = L->h;
    h.bound0 = bound0;
    h.i0 = ipix;
    h.nend = npix;
    h.idet0 = idet;
    h.alpha = parea;
    h.flags = 0;
    if (ipix >= npix || idet >= maxn) {
        h.npiece = 0;
        h.endv = bound0;
    } else {
        const float b0 = FADD(FMUL((float)(ipix + 1), pint), p0);
        int fl = 0;
        h.npiece = dd_build_pieces(b0, pint, ipix, npix, L->p, &fl);
        h.flags = fl;
        h.endv = L->p[h.npiece - 1].Q;
        dd_build_slots(L->p, h.npiece, L->slot);
    }
}

// ---------------------------------------------------------------------------
// Drifted pixel boundaries of a record
// ---------------------------------------------------------------------------
// Piece holding boundary index i, starting from hint p.
DD_HD int dd3_piece_at(const DdLine *L, int i, int p) {
    const int np = L->h.npiece;
    while (p < np - 1 && i > L->p[p].gb) p++;
    while (p > 0 && i <= L->p[p - 1].gb) p--;
    return p;
}

// Boundary i (upper boundary of pixel i); p is the piece hint, updated.
DD_HD float dd3_bnd(const DdLine *L, int i, int *p) {
    *p = dd3_piece_at(L, i, *p);
    const DdPiece P = L->p[*p];
    return FADD(P.Q, FMUL((float)(i - P.gb), P.dl));
}

// First pixel j >= i0 whose upper boundary exceeds u (nend if none); p
// receives the piece of boundary j (or of the last boundary).
DD_HD int dd3_pixel_of(const DdLine *L, float u, int *p) {
    const int i0 = L->h.i0, nend = L->h.nend;
    int pp, j;
    float rr;
    dd_locate(L, u, &pp, &j, &rr);   // estimate: b_{j-1} <= u < b_j
    if (j < i0) j = i0;
    // correct the estimate against the exact boundaries
    for (int it = 0; it < 4 && j < nend; it++) {
        if (u >= dd3_bnd(L, j, &pp)) j++;
        else break;
    }
    for (int it = 0; it < 4 && j > i0; it++) {
        if (u < dd3_bnd(L, j - 1, &pp)) j--;
        else break;
    }
    // fall back to a bisection if the estimate was far off
    const bool ok_hi = (j >= nend) || (u < dd3_bnd(L, j, &pp));
    const bool ok_lo = (j == i0) || (u >= dd3_bnd(L, j - 1, &pp));
    if (!(ok_hi && ok_lo)) {
        int lo = i0, hi = nend;   // answer in [lo, hi]
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (u < dd3_bnd(L, mid, &pp)) hi = mid;
            else lo = mid + 1;
        }
        j = lo;
    }
    *p = (j < nend) ? dd3_piece_at(L, j, pp) : L->h.npiece - 1;
    return j;
}

// ---------------------------------------------------------------------------
// Closed-form z cells.  The reference's z walk starts each (line, column, row)
// cell at bz0 = max(p0z, rp0) in slice is0 = floor((bz0 - p0z) / pintz), takes
// is0 * pintz + p0z + pintz as the first slice top and then adds pintz once per
// further slice (1-3 slices, so FP32 drift stays at the ulp level;
// ConeFlatDisCUDA3d.cu:131-152).  Here the top of slice s is always
// dd3_zb(s + 1) -- the reference's own formula for the first top -- and the
// width of (row, slice) is the overlap of the row interval [bz0, bz1] with
// [dd3_zb(s), dd3_zb(s + 1)].  Forward and adjoint evaluate the same
// expression, so they stay exact transposes.
// ---------------------------------------------------------------------------
DD_HD float dd3_zb(float p0z, float pintz, int s) { return FADD(FMUL((float)s, pintz), p0z); }

DD_HD float dd3_cell(float bz0, float bz1, float zlo, float zhi) {
    const float lo = bz0 > zlo ? bz0 : zlo;
    const float hi = bz1 < zhi ? bz1 : zhi;
    return hi > lo ? FSUB(hi, lo) : 0.0f;
}

// First slice a row interval starting at bz0 can meet (one below the
// estimate, so that no slice with a positive width is skipped).
DD_HD int dd3_slice_first(float bz0, float p0z, float pintz) {
    int s = (int)floorf(dd3_approx_div(FSUB(bz0, p0z), pintz)) - 1;
    return s < 0 ? 0 : s;
}

// ---------------------------------------------------------------------------
// Sorted column search: first k in [klo, khi) with dp[k+1] > u (khi if
// none).  An analytic estimate from the detector geometry, corrected against
// the exact boundary table, with a bisection as the fallback.
// ---------------------------------------------------------------------------
DD_HD int dd3_col_of(int geom, const dd_geom3d *g, const DdView3 *w, const float *dp, float u, int klo,
                     int khi) {
    if (klo >= khi) return khi;
    const int C = g->num_col;
    float kf;
    if (geom == DD_GEOM3_CONE_FLAT) {
        const float R = g->iso_source;
        const float t = w->xb ? dd3_approx_div(R * u * w->c, R + u * w->s) : dd3_approx_div(R * u * w->s, R - u * w->c);
        const float q = dd3_approx_div(t - w->vbs, w->vds);
        kf = w->flip ? (float)C * 0.5f - q : q + (float)C * 0.5f;
    } else {
        float ang = w->xb ? atan2f(u - w->srcx, w->srcy)
                          : 1.5707963267948966f - atanf(dd3_approx_div(u - w->srcy, w->srcx));
        const float base = w->view + w->colshift;
        ang += 3.14159265358979f * rintf((base - ang) * 0.3183098861837907f);
        const float q = dd3_approx_div(ang - base, w->colsz);
        kf = w->flip ? (float)C * 0.5f - q : q + (float)C * 0.5f;
    }
    int k = klo;
    if (kf == kf) k = (int)floorf(fminf(fmaxf(kf, -1.0e6f), 1.0e6f));
    if (k < klo) k = klo;
    if (k > khi - 1) k = khi - 1;
    for (int it = 0; it < 4 && k > klo && dp[k] > u; it++) k--;
    for (int it = 0; it < 4 && k < khi && dp[k + 1] <= u; it++) k++;
    const bool ok = (k == khi || dp[k + 1] > u) && (k == klo || dp[k] <= u);
    if (!ok) {
        int lo = klo, hi = khi;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (dp[mid + 1] > u) hi = mid;
            else lo = mid + 1;
        }
        k = lo;
    }
    return k;
}

// ---------------------------------------------------------------------------
// Segments of one column (forward-type kernels)
// ---------------------------------------------------------------------------
struct DdColWalk {
    int j, p;
    float plo, CL, CH;
};

// kk = column index within its walk block; dp = the view's boundary table.
DD_HD bool dd3_colwalk_init(const DdLine *L, const float *dp, int k, int kk, DdColWalk *cw) {
    const DdLineHdr h = L->h;
    if (h.npiece == 0 || kk < h.idet0) return false;
    cw->CL = (kk == h.idet0) ? h.bound0 : dp[k];
    cw->CH = dp[k + 1];
    int p;
    const int j = dd3_pixel_of(L, cw->CL, &p);
    if (j >= h.nend) return false;
    cw->j = j;
    cw->p = p;
    if (j == h.i0) {
        cw->plo = h.bound0;
    } else {
        int q = p;
        cw->plo = dd3_bnd(L, j - 1, &q);
    }
    return true;
}

// Next segment (pixel j, width w) of the column; false when done.
DD_HD bool dd3_colwalk_next(const DdLine *L, DdColWalk *cw, int *j, float *w) {
    const int nend = L->h.nend;
    while (cw->j < nend && cw->plo < cw->CH) {
        const float phi = dd3_bnd(L, cw->j, &cw->p);
        const float hi = phi < cw->CH ? phi : cw->CH;
        const float lo = cw->plo > cw->CL ? cw->plo : cw->CL;
        const int jj = cw->j;
        cw->plo = phi;
        cw->j++;
        if (hi > lo) {
            *j = jj;
            *w = FSUB(hi, lo);
            return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// Segments of one pixel in one walk block (adjoint-type kernels)
// ---------------------------------------------------------------------------
struct DdPixWalk {
    int k, klo, khi;
    float PL, PH, bound0;
};

DD_HD bool dd3_pixwalk_init(int geom, const dd_geom3d *g, const DdView3 *w, const DdLine *L, const float *dp,
                            int cc, int j, DdPixWalk *pw) {
    const DdLineHdr h = L->h;
    if (h.npiece == 0 || j < h.i0 || j >= h.nend) return false;
    const int C = g->num_col;
    const int c0 = cc * DD3_CHUNK;
    const int maxn = (C - c0 < DD3_CHUNK) ? C - c0 : DD3_CHUNK;
    const DdPiece P0 = L->p[0];
    int p = dd_piece_of_index(L, j, FADD(P0.Q, FMUL((float)(j - P0.gb), P0.dl)));
    pw->PH = dd3_bnd(L, j, &p);
    pw->PL = (j == h.i0) ? h.bound0 : dd3_bnd(L, j - 1, &p);
    pw->bound0 = h.bound0;
    pw->klo = c0 + h.idet0;
    pw->khi = c0 + maxn;
    // quick rejection: the block's columns end before the pixel starts
    if (!(dp[pw->khi] > pw->PL)) return false;
    pw->k = dd3_col_of(geom, g, w, dp, pw->PL, pw->klo, pw->khi);
    return pw->k < pw->khi;
}

DD_HD bool dd3_pixwalk_next(const float *dp, DdPixWalk *pw, int *k, float *wd) {
    while (pw->k < pw->khi) {
        const float CL = (pw->k == pw->klo) ? pw->bound0 : dp[pw->k];
        if (!(CL < pw->PH)) {
            pw->k = pw->khi;
            return false;
        }
        const float CH = dp[pw->k + 1];
        const float hi = pw->PH < CH ? pw->PH : CH;
        const float lo = pw->PL > CL ? pw->PL : CL;
        const int kk = pw->k;
        pw->k++;
        if (hi > lo) {
            *k = kk;
            *wd = FSUB(hi, lo);
            return true;
        }
    }
    return false;
}

// Weight factor of one segment for the operator family: the width itself
// (Proj / ProjTrans), width / pixel area (DD backprojector), times (flat) or
// divided by (arc, spiral) the FBP weight at the pixel centre (weighted
// variants).  ConeFlatDisCUDA3d.cu:630-640.
DD_HD float dd3_coef(int geom, int family, const dd_geom3d *g, const DdView3 *w, float lpos, int j, float width,
                     float parea) {
    if (family == 0) return width;
    float c = FDIV(width, parea);
    if (family == 2) {
        float px, py;
        dd3_pix_centre(g, w, lpos, j, &px, &py);
        if (geom == DD_GEOM3_CONE_FLAT) c = FMUL(c, dd_cw_flat(w->srcx, w->srcy, px, py, w->iso));
        else c = FDIV(c, dd_cw_arc(w->srcx, w->srcy, px, py));
    }
    return c;
}

// ---------------------------------------------------------------------------
// Rows of one column that may meet a slice (adjoint-type kernels)
// ---------------------------------------------------------------------------
// rowz: the view's row table {row0z, row1z} x R.  Returns the first row
// whose upper boundary on the line plane may exceed zlo - margin; callers
// walk rows upward until the lower boundary passes the slice top.
DD_HD int dd3_row_first(int geom, const DdView3 *w, const float *rowz, int R, float mag, float zlo,
                        float margin) {
    const float zeta = (geom == DD_GEOM3_SPIRAL) ? dd3_approx_div(zlo - w->srcz, mag) + w->srcz
                                                 : dd3_approx_div(zlo, mag);
    int r = 0;
    if (w->rzB > 0.0f) {
        const float rf = dd3_approx_div(zeta - w->rzA, w->rzB);
        if (rf == rf) r = (int)floorf(fminf(fmaxf(rf, -1.0f), (float)R)) - 1;
    }
    if (r < 0) r = 0;
    if (r > R - 1) r = R - 1;
    for (int it = 0; it < 64 && r > 0; it++) {
        float a, b;
        dd3_rp(geom, w, mag, rowz[2 * (r - 1)], rowz[2 * (r - 1) + 1], &a, &b);
        if (b > zlo - margin) r--;
        else break;
    }
    return r;
}

// Conservative test whether volume slices with z in [zs0, zs1] can meet any
// detector row of this view on lines whose magnification lies in [mlo, mhi]
// (rows span [zr0, zr1] before magnification).
DD_HD bool dd3_slab_lit(const DdView3 *w, float mlo, float mhi, float zs0, float zs1, float zr0, float zr1) {
    if (!(mlo > 0.0f) || !(w->magmin > 0.0f)) return true;   // source inside the volume: no bound
    const float rmin = w->magmin / mhi, rmax = w->magmax / mlo;
    const float a = zr1 - w->srcz, b = zr0 - w->srcz;
    const float top = (a >= 0.0f) ? rmax * a : rmin * a;      // highest row boundary
    const float bot = (b >= 0.0f) ? rmin * b : rmax * b;      // lowest row boundary
    const float tol = 1e-3f * (fabsf(top) + fabsf(bot)) + 1e-3f;
    return (zs0 - w->srcz) < top + tol && (zs1 - w->srcz) > bot - tol;
}
