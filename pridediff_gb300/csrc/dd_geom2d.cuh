// 2-D view and line set-up for parallel, fan-flat and fan-arc DD projection.
//
// Reproduces the per-view and per-line arithmetic of deeprecon's CPU
// projectors (ParaDisCPU2d.cpp, FanFlatDisCPU2d.cpp, FanArcDisCPU2d.cpp) with
// the same FP32/FP64 promotions, so that the detector boundary table, the
// start of every walk and the drifted pixel boundaries are bit-identical to
// the ones the reference visits.  Citations point at the x-branch line of
// each step; the y-branch lines follow the same pattern a few lines below.
#pragma once

#include "dd_geom.cuh"
#include "../../include/pridediff_dd.h"

enum { DD_GEOM_PARA = 0, DD_GEOM_FLAT = 1, DD_GEOM_ARC = 2 };

// Per-view scalars.  Para: ParaDisCPU2d.cpp:46-61, :105-113.
// Flat: FanFlatDisCPU2d.cpp:62-71, :94.  Arc: FanArcDisCPU2d.cpp:69-76.
DD_HD void dd_view2_scalars(int geom, const dd_geom2d *g, float view, DdView2 *vw) {
    const int D = g->num_det, W = g->width, H = g->height;
    const float ds = g->det_size, R = g->iso_source, SDD = g->source_detector;
    const float bin = g->bin_shift;
    const float s = (float)sin((double)view);
    const float c = (float)cos((double)view);
    vw->s = s;
    vw->c = c;
    vw->xb = FMUL(c, c) > 0.5f;
    vw->flip = vw->xb ? (c < 0.0f) : (s < 0.0f);
    vw->srcx = FMUL(-s, R);
    vw->srcy = FMUL(c, R);
    vw->det0 = vw->di = vw->det0xy = 0.0f;
    vw->pad = 0.0f;
    // image extent on the walked axis (ParaDisCPU2d.cpp:57, :110; FanFlat :92-93, :161-162)
    if (vw->xb) {
        vw->axis0 = (float)DADD(DMUL(-W / 2.0, (double)g->pix_x), (double)g->pix_xshift);
        vw->axis1 = (float)DADD(DMUL(W / 2.0, (double)g->pix_x), (double)g->pix_xshift);
    } else {
        vw->axis0 = (float)DADD(DMUL(-H / 2.0, (double)g->pix_y), (double)g->pix_yshift);
        vw->axis1 = (float)DADD(DMUL(H / 2.0, (double)g->pix_y), (double)g->pix_yshift);
    }
    if (geom == DD_GEOM_PARA) {
        const float t = vw->xb ? c : s;
        const double half = (t >= 0.0f) ? -D / 2.0 : D / 2.0;
        vw->det0 = (float)DDIV(DADD(DMUL(half, (double)ds), (double)bin), (double)t);
        vw->di = (float)DDIV((double)ds, fabs((double)t));
    } else if (geom == DD_GEOM_FLAT) {
        const float vds = FMUL(FDIV(R, SDD), ds), vbs = FMUL(FDIV(R, SDD), bin);
        const double u = vw->flip ? DADD(DMUL(D / 2.0, (double)vds), (double)vbs)
                                  : DADD(DMUL(-D / 2.0, (double)vds), (double)vbs);
        vw->det0xy = vw->xb ? (float)DMUL(u, (double)c) : (float)DMUL(u, (double)s);
        vw->di = (float)DMUL((double)vds, fabs((double)(vw->xb ? c : s)));
    }
}

// Sorted detector boundary k (0..D) on the axis, fan beams.
// Flat: FanFlatDisCPU2d.cpp:73-83.  Arc: FanArcDisCPU2d.cpp:77-86.
DD_HD float dd_view2_boundary(int geom, const dd_geom2d *g, float view, const DdView2 *vw, int k) {
    const int D = g->num_det;
    const float ds = g->det_size, R = g->iso_source, SDD = g->source_detector;
    const float bin = g->bin_shift;
    if (geom == DD_GEOM_FLAT) {
        const float vds = FMUL(FDIV(R, SDD), ds), vbs = FMUL(FDIV(R, SDD), bin);
        const double u = vw->flip ? DADD(DMUL(DSUB(D / 2.0, (double)k), (double)vds), (double)vbs)
                                  : DADD(DMUL(DSUB((double)k, D / 2.0), (double)vds), (double)vbs);
        const float dx = (float)DMUL(u, (double)vw->c), dy = (float)DMUL(u, (double)vw->s);
        return vw->xb ? dd_map2x(vw->srcx, vw->srcy, dx, dy) : dd_map2y(vw->srcx, vw->srcy, dx, dy);
    }
    const double a = vw->flip
        ? DADD(DADD(DMUL(DSUB(D / 2.0, (double)k), (double)ds), (double)bin), (double)view)
        : DADD(DADD(DMUL(DSUB((double)k, D / 2.0), (double)ds), (double)bin), (double)view);
    const float ang = (float)a;
    return vw->xb ? (float)DADD((double)vw->srcx, DMUL((double)vw->srcy, tan((double)ang)))
                  : (float)DADD((double)vw->srcy, DDIV((double)vw->srcx, tan((double)ang)));
}

// Per-bin scale of Proj / ProjTrans between sorted boundaries d0 < d1
// (CoefTemp, FanFlatDisCPU2d.cpp:84-90).
DD_HD float dd_view2_bcoef(const dd_geom2d *g, const DdView2 *vw, float d0, float d1) {
    const float pix = vw->xb ? g->pix_y : g->pix_x;
    const float src_a = vw->xb ? vw->srcx : vw->srcy, src_b = vw->xb ? vw->srcy : vw->srcx;
    const float mid = (float)DSUB(DDIV((double)FADD(d1, d0), 2.0), (double)src_a);
    return FDIV(pix, FMUL(FSUB(d1, d0), dd_tricos2(mid, src_b)));
}

// Whole-view set-up on one thread (host checks): scalars, D+1 boundaries and
// D per-bin scales (dp/bcoef unused for the parallel beam).
DD_HD void dd_view2_setup(int geom, const dd_geom2d *g, float view, DdView2 *vw, float *dp,
                          float *bcoef) {
    dd_view2_scalars(geom, g, view, vw);
    if (geom == DD_GEOM_PARA) return;
    for (int k = 0; k <= g->num_det; k++) dp[k] = dd_view2_boundary(geom, g, view, vw, k);
    for (int k = 0; k < g->num_det; k++) bcoef[k] = dd_view2_bcoef(g, vw, dp[k], dp[k + 1]);
}

// Start of the walk of one line: first pixel boundary p0 and pixel pitch
// pint on the projection axis, walk start bound0, first pixel i0 and first
// detector bin idet0 (ParaDisCPU2d.cpp:62-77, FanFlatDisCPU2d.cpp:95-113,
// FanArcDisCPU2d.cpp:97-120).
struct DdLineStart {
    float p0, pint, bound0;
    int i0, idet0;
};

DD_HD void dd_line2_start(int geom, const dd_geom2d *g, float view, const DdView2 *vw,
                          const float *dp, int line, DdLineStart *st) {
    const int W = g->width, H = g->height, D = g->num_det;
    const int xb = vw->xb;
    const int npix = xb ? W : H;
    // centre of the walked line: row y (xb) or column x
    const float lpos = xb
        ? (float)DADD(DMUL(DSUB(DSUB(H / 2.0, (double)line), 0.5), (double)g->pix_y), (double)g->pix_yshift)
        : (float)DADD(DMUL(DADD(DSUB((double)line, W / 2.0), 0.5), (double)g->pix_x), (double)g->pix_xshift);
    float p0, pint;
    if (geom == DD_GEOM_PARA) {
        p0 = xb ? FADD(FMUL(FDIV(vw->s, vw->c), lpos), vw->axis0)
                : FADD(FMUL(FDIV(vw->c, vw->s), lpos), vw->axis0);
        pint = xb ? g->pix_x : g->pix_y;
    } else {
        float p1;
        if (xb) {
            p0 = dd_map2x(vw->srcx, vw->srcy, vw->axis0, lpos);
            p1 = dd_map2x(vw->srcx, vw->srcy, vw->axis1, lpos);
        } else {
            p0 = dd_map2y(vw->srcx, vw->srcy, lpos, vw->axis0);
            p1 = dd_map2y(vw->srcx, vw->srcy, lpos, vw->axis1);
        }
        pint = FDIV(FSUB(p1, p0), (float)npix);
    }
    // start rule
    float bound0;
    int i0, idet0;
    if (geom == DD_GEOM_ARC) {
        // FanArcDisCPU2d.cpp:102-116 (x) and :172-186 (y)
        const float base = FADD(g->bin_shift, view);
        float tan0, tan1;
        if (xb) {
            const float dxs = FSUB(vw->srcx, p0);
            tan0 = (dxs == 0.0f) ? 1e10f : FDIV(vw->srcy, dxs);
            tan1 = (base == 0.0f) ? 1e10f : (float)DDIV(-1.0, tan((double)base));
        } else {
            tan0 = FDIV(FSUB(vw->srcy, p0), vw->srcx);
            tan1 = (float)DDIV(-1.0, tan((double)base));
        }
        const float q = FDIV(FSUB(tan0, tan1), FADD(1.0f, FMUL(tan0, tan1)));
        const float delta = (float)atan((double)q);
        const float flag = vw->flip ? -1.0f : 1.0f;
        idet0 = (int)floor(DADD(D / 2.0, (double)FDIV(FMUL(delta, flag), g->det_size)));
        if (idet0 < 0) {
            bound0 = dp[0];
            i0 = dd_ifloor(FDIV(FSUB(bound0, p0), pint));
            idet0 = 0;
        } else {
            bound0 = p0;
            i0 = 0;
        }
    } else {
        const float d0 = (geom == DD_GEOM_PARA) ? vw->det0 : dp[0];
        bound0 = (float)fmax((double)p0, (double)d0);
        if (p0 == bound0) {
            i0 = 0;
            if (geom == DD_GEOM_PARA) {
                idet0 = dd_ifloor(FDIV(FSUB(bound0, d0), vw->di));
            } else {
                // FanFlatDisCPU2d.cpp:105-107 / :174-176
                const float back = xb
                    ? FDIV(FMUL(vw->srcy, bound0),
                           FADD(FDIV(FMUL(FSUB(bound0, vw->srcx), vw->s), vw->c), vw->srcy))
                    : FDIV(FMUL(vw->srcx, bound0),
                           FADD(FDIV(FMUL(FSUB(bound0, vw->srcy), vw->c), vw->s), vw->srcx));
                idet0 = dd_ifloor(FDIV(FSUB(back, vw->det0xy), vw->di));
            }
        } else {
            i0 = dd_ifloor(FDIV(FSUB(bound0, p0), pint));
            idet0 = 0;
        }
    }
    if (idet0 < 0) idet0 = 0;   // the reference indexes out of bounds there
    if (i0 < 0) i0 = 0;
    st->p0 = p0;
    st->pint = pint;
    st->bound0 = bound0;
    st->i0 = i0;
    st->idet0 = idet0;
}

// Per-line set-up: start of the walk and the drifted pixel boundaries.
// `L` receives the pixel-side record; for the parallel beam `Ld` receives the
// drifted detector-side record (may be NULL otherwise).
DD_HD void dd_line2_setup(int geom, const dd_geom2d *g, float view, const DdView2 *vw,
                          const float *dp, int line, DdLine *L, DdLine *Ld) {
    const int D = g->num_det;
    const int npix = vw->xb ? g->width : g->height;
    DdLineStart st;
    dd_line2_start(geom, g, view, vw, dp, line, &st);
    const float p0 = st.p0, pint = st.pint, bound0 = st.bound0;
    const int i0 = st.i0, idet0 = st.idet0;
    DdLineHdr &h = L->h;
    h.bound0 = bound0;
    h.i0 = i0;
    h.nend = npix;
    h.idet0 = idet0;
    h.flags = 0;
    // DD-BP per-line scale: ParaDisCPU2d.cpp:202, FanFlatDisCPU2d.cpp:478, FanArcDisCPU2d.cpp:480
    if (geom == DD_GEOM_PARA) h.alpha = FDIV(g->det_size, pint);
    else if (geom == DD_GEOM_FLAT) h.alpha = FDIV(FMUL(FDIV(g->iso_source, g->source_detector), g->det_size), pint);
    else h.alpha = FDIV(FMUL(g->iso_source, g->det_size), pint);
    if (i0 >= npix || idet0 >= D) {
        h.npiece = 0;
        h.endv = bound0;
    } else {
        // first upper boundary: (idxcol + 1) * PixInterval + Point0Proj
        const float b0 = FADD(FMUL((float)(i0 + 1), pint), p0);
        int fl = 0;
        h.npiece = dd_build_pieces(b0, pint, i0, npix, L->p, &fl);
        h.flags = fl;
        h.endv = L->p[h.npiece - 1].Q;
        dd_build_slots(L->p, h.npiece, L->slot);
    }
    if (Ld) {
        // parallel beam: detector boundaries also advance by repeated FP32
        // addition (ParaDisCPU2d.cpp:76, :100)
        DdLineHdr &hd = Ld->h;
        hd.bound0 = bound0;
        hd.i0 = idet0;
        hd.nend = D;
        hd.idet0 = i0;
        hd.alpha = h.alpha;
        hd.flags = 0;
        if (h.npiece == 0) {
            hd.npiece = 0;
            hd.endv = bound0;
        } else {
            const float d1 = FADD(FMUL((float)(idet0 + 1), vw->di), vw->det0);
            int fl = 0;
            hd.npiece = dd_build_pieces(d1, vw->di, idet0, D, Ld->p, &fl);
            hd.flags = fl;
            hd.endv = Ld->p[hd.npiece - 1].Q;
            dd_build_slots(Ld->p, hd.npiece, Ld->slot);
        }
    }
}

// ---------------------------------------------------------------------------
// System matrix of one walked line: the merge walk exactly as deeprecon's
// CPU builders run it (GetSysMatrixPara2dKernel, ParaDisCPU2d.cpp:488-612;
// GetSysMatrixFanFlat2dKernel, FanFlatDisCPU2d.cpp:1048-1216;
// GetSysMatrixFanArc2dKernel, FanArcDisCPU2d.cpp:1057-), sequential FP32
// recurrences included: one entry per step, row = view * D + detector bin
// (reversed when the detector is flipped), column = pixel index in the image,
// value = step width x bin scale.  With rows == NULL the entries are only
// counted.  Returns the number of entries.  bcoef: the view's per-bin scales
// (fan beams); dp: its boundary table (fan beams).
// ---------------------------------------------------------------------------
DD_HD long long dd_line2_sysmat(int geom, const dd_geom2d *g, float view, const DdView2 *vw, const float *dp,
                                const float *bcoef, int v, int line, long long *rows, long long *cols,
                                float *vals) {
    const int W = g->width, H = g->height, D = g->num_det;
    const int xb = vw->xb;
    const int npix = xb ? W : H, nline = xb ? H : W;
    if (line < 0 || line >= nline) return 0;
    DdLineStart st;
    dd_line2_start(geom, g, view, vw, dp, line, &st);
    float b = st.bound0;
    int ipix = st.i0, idet = st.idet0;
    float point1 = FADD(FMUL((float)(ipix + 1), st.pint), st.p0);
    float det1 = 0.0f;
    if (geom == DD_GEOM_PARA) det1 = FADD(FMUL((float)(idet + 1), vw->di), vw->det0);
    else if (idet < D) det1 = dp[idet + 1];
    const float pbeta = xb ? FDIV(g->pix_y, g->det_size) : FDIV(g->pix_x, g->det_size);
    long long n = 0;
    while (ipix < npix && idet < D) {
        const bool step_pix = point1 < det1;
        if (rows) {
            const float w = FSUB(step_pix ? point1 : det1, b);
            rows[n] = (long long)v * D + (vw->flip ? D - 1 - idet : idet);
            cols[n] = xb ? (long long)line * W + ipix : (long long)(H - 1 - ipix) * W + line;
            vals[n] = FMUL(w, geom == DD_GEOM_PARA ? pbeta : bcoef[idet]);
        }
        n++;
        if (step_pix) {
            b = point1;
            ipix++;
            point1 = FADD(point1, st.pint);
        } else {
            b = det1;
            idet++;
            if (geom == DD_GEOM_PARA) det1 = FADD(det1, vw->di);
            else if (idet < D) det1 = dp[idet + 1];
        }
    }
    return n;
}
