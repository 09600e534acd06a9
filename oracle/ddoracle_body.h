/*
 * Body of the CPU oracle, compiled twice by ddoracle.c: once with T = float
 * (a faithful restatement of deeprecon's FP32 arithmetic, the parity oracle
 * and the CPU baseline "port") and once with T = double (the FP64 oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links this code.
 *
 * The algorithm is deeprecon's distance-driven (DD) merge walk.  deeprecon
 * repeats the walk in 18 copy-pasted kernels (6 operators x 3 geometries in
 * cpu/dis2d/<geom>DisCPU2d.cpp, and 6 x 3 more in cuda/dis3d/<geom>DisCUDA3d.cu); here ONE walk per
 * dimensionality is parameterised by a per-view geometry record and by the
 * operator.  The arithmetic of each step (which values are rounded to FP32
 * and when, the incremental boundary updates, the start-index rules) follows
 * the reference line by line so that the FP32 instantiation reproduces the
 * reference's rounding; citations are given at each step.
 *
 * Expects: T (scalar type), FN(name) (name mangler).
 */

/* ------------------------------------------------------------------------ */
/* 2-D                                                                       */
/* ------------------------------------------------------------------------ */

/* Per-view geometry of one 2-D view, in "axis" coordinates: every boundary
 * is projected (through the source for fan beams) onto the x axis (xb = 1,
 * image rows are walked) or the y axis (xb = 0, image columns are walked,
 * rows counted from the bottom). */
typedef struct {
    int xb;          /* cos^2 > 0.5: project to x and walk rows             */
    int flip;        /* detector index reversed (cos < 0 resp. sin < 0)     */
    T s, c;          /* sin, cos of the view angle (FP32-rounded for T=f)   */
    T srcx, srcy;    /* source position (fan)                               */
    T *dp;           /* D+1 sorted detector boundaries on the axis (fan)    */
    T *bcoef;        /* D per-bin scale of Proj / ProjTrans (fan)           */
    /* parallel beam: uniform boundaries Det0 + k*DI                         */
    T det0, di;
    /* fan-flat start rule                                                   */
    T det0xy;        /* x (resp. y) of virtual-detector boundary 0          */
    int flag;        /* fan-arc: +1 / -1                                     */
} FN(view2);

/* Apply one walk segment to the output (the body of the reference's inner
 * batch loop, e.g. FanFlatDisCPU2d.cpp:116-122, :300-310, :495-506,
 * :689-696).  `coef` already holds segment-length x operator scale. */
static inline void FN(emit2)(int op, const T *in, T *out, int batch,
                             long long pix, long long pixstride,
                             long long det, long long detstride, T coef,
                             T wgt, int use_w, int arcw, int atomic)
{
    for (int b = 0; b < batch; b++) {
        if (op == DDO_PROJ || op == DDO_BPROJ_T || op == DDO_BPROJ_TW) {
            T v = in[b * pixstride + pix] * coef;
            if (use_w) v = arcw ? v / wgt : v * wgt;
            out[b * detstride + det] += v;   /* bin owned by this thread */
        } else {
            T v = in[b * detstride + det] * coef;
            if (use_w) v = arcw ? v / wgt : v * wgt;
            if (atomic) FN(atomic_add)(out + b * pixstride + pix, v);
            else out[b * pixstride + pix] += v;
        }
    }
}

static T FN(map2x)(T sx, T sy, T px, T py) { return (sx * py - sy * px) / (py - sy); }
static T FN(map2y)(T sx, T sy, T px, T py) { return (sy * px - sx * py) / (px - sx); }
/* |b| / sqrt(a^2+b^2): FanFlatDisCPU2d.cpp:24-26 (the reference promotes the
 * square root to double and rounds the quotient on return). */
static T FN(tricos2)(T a, T b) { return (T)(fabs((double)b) / sqrt((double)(a * a + b * b))); }
/* FanFlatDisCPU2d.cpp:19-22 */
static T FN(cw_flat)(T sx, T sy, T px, T py, T r)
{
    T d = (sx * px + sy * py) / r;
    return r * r / ((r - d) * (r - d));
}
/* FanArcDisCPU2d.cpp:27-29 */
static T FN(cw_arc)(T sx, T sy, T px, T py)
{
    return (sx - px) * (sx - px) + (sy - py) * (sy - py);
}

/* Per-view set-up.  Para: ParaDisCPU2d.cpp:46-61, :105-113.
 * Flat: FanFlatDisCPU2d.cpp:62-94, :141-163.  Arc: FanArcDisCPU2d.cpp:69-94,
 * :146-166. */
static void FN(setup_view2)(const ddo_geom2 *g, int geom, T view, FN(view2) *vw)
{
    const int D = g->nd;
    const T ds = (T)g->det_size, R = (T)g->iso_source, SDD = (T)g->source_detector;
    const T bin = (T)g->bin_shift;
    vw->s = (T)sin((double)view);
    vw->c = (T)cos((double)view);
    const T s = vw->s, c = vw->c;
    /* The x/y branch is a discrete property of the reference operator: it is
     * decided from the FP32-rounded cosine at every precision, so that the
     * FP64 instantiation evaluates the same discretisation as the FP32 one
     * (views at exactly 45 degrees sit on the cos^2 = 0.5 boundary). */
    {
        const float cf = (float)cos((double)view), sf = (float)sin((double)view);
        vw->xb = (cf * cf > 0.5);
        vw->flip = vw->xb ? (cf < 0) : (sf < 0);
    }
    vw->srcx = -s * R;
    vw->srcy = c * R;
    vw->flag = vw->flip ? -1 : 1;
    vw->det0 = vw->di = vw->det0xy = 0;
    if (geom == DDO_PARA) {
        const T t = vw->xb ? c : s;
        vw->det0 = (T)(((t >= 0 ? -D / 2.0 : D / 2.0) * ds + bin) / t);
        vw->di = (T)(ds / fabs((double)t));
        return;
    }
    if (geom == DDO_FLAT) {
        const T vds = R / SDD * ds, vbs = R / SDD * bin;
        for (int k = 0; k <= D; k++) {
            double u = vw->flip ? (D / 2.0 - k) * vds + vbs : (k - D / 2.0) * vds + vbs;
            T dx = (T)(u * c), dy = (T)(u * s);
            if (k == 0) vw->det0xy = vw->xb ? dx : dy;
            vw->dp[k] = vw->xb ? FN(map2x)(vw->srcx, vw->srcy, dx, dy)
                               : FN(map2y)(vw->srcx, vw->srcy, dx, dy);
        }
        vw->di = (T)(vds * fabs((double)(vw->xb ? c : s)));
    } else { /* DDO_ARC */
        for (int k = 0; k <= D; k++) {
            T ang = (T)(vw->flip ? (D / 2.0 - k) * ds + bin + view : (k - D / 2.0) * ds + bin + view);
            vw->dp[k] = vw->xb ? (T)(vw->srcx + vw->srcy * tan((double)ang))
                               : (T)(vw->srcy + vw->srcx / tan((double)ang));
        }
    }
    const T pix = vw->xb ? (T)g->pix_y : (T)g->pix_x;
    for (int k = 0; k < D; k++) {
        T mid = (T)((vw->dp[k + 1] + vw->dp[k]) / 2.0 - (vw->xb ? vw->srcx : vw->srcy));
        vw->bcoef[k] = pix / ((vw->dp[k + 1] - vw->dp[k]) *
                              FN(tricos2)(mid, vw->xb ? vw->srcy : vw->srcx));
    }
}

/* Walk every image line of one view and apply `op` (the per-line part of
 * ParaDisCPU2d.cpp:62-103 / :115-156, FanFlatDisCPU2d.cpp:95-139 / :164-208,
 * FanArcDisCPU2d.cpp:97-146 and their transposes / backprojectors). */
static void FN(walk_view2)(const ddo_geom2 *g, int geom, int op, int v, T view,
                           const FN(view2) *vw, const T *in, T *out, int batch,
                           int atomic)
{
    const int W = g->width, H = g->height, D = g->nd, V = g->nv;
    const T sx = (T)g->pix_x, sy = (T)g->pix_y, ds = (T)g->det_size;
    const T R = (T)g->iso_source, SDD = (T)g->source_detector;
    const T pxs = (T)g->pix_xshift, pys = (T)g->pix_yshift, bin = (T)g->bin_shift;
    const T s = vw->s, c = vw->c;
    const int xb = vw->xb;
    const int nline = xb ? H : W, npix = xb ? W : H;
    const long long pixstride = (long long)W * H, detstride = (long long)V * D;
    const int fbp = (op == DDO_BPROJ_W || op == DDO_BPROJ_TW);
    const int trans_scale = (op == DDO_PROJ || op == DDO_PROJ_T);   /* uses bcoef */

    /* para scales: ParaDisCPU2d.cpp:60, :113, :202, :263 */
    T para_coef = 0;
    if (geom == DDO_PARA) {
        const T pint = xb ? sx : sy;
        if (trans_scale) para_coef = (xb ? sy : sx) / ds;
        else para_coef = ds / pint;
    }
    const T axis0 = xb ? (T)(-W / 2.0 * sx + pxs) : (T)(-H / 2.0 * sy + pys);
    const T axis1 = xb ? (T)(W / 2.0 * sx + pxs) : (T)(H / 2.0 * sy + pys);

    for (int line = 0; line < nline; line++) {
        /* line position: row centre y (xb) or column centre x */
        const T lpos = xb ? (T)((H / 2.0 - line - 0.5) * sy + pys)
                          : (T)((line - W / 2.0 + 0.5) * sx + pxs);
        T p0, pint;
        if (geom == DDO_PARA) {
            p0 = xb ? s / c * lpos + axis0 : c / s * lpos + axis0;
            pint = xb ? sx : sy;
        } else {
            T p1;
            if (xb) {
                p0 = FN(map2x)(vw->srcx, vw->srcy, axis0, lpos);
                p1 = FN(map2x)(vw->srcx, vw->srcy, axis1, lpos);
            } else {
                p0 = FN(map2y)(vw->srcx, vw->srcy, lpos, axis0);
                p1 = FN(map2y)(vw->srcx, vw->srcy, lpos, axis1);
            }
            pint = (p1 - p0) / (T)npix;
        }
        /* DD-BP scale per line: FanFlatDisCPU2d.cpp:478, FanArcDisCPU2d.cpp:480 */
        T line_coef = para_coef;
        if (geom == DDO_FLAT && !trans_scale) line_coef = (R / SDD * ds) / pint;
        if (geom == DDO_ARC && !trans_scale) line_coef = (R * ds) / pint;

        /* start indices */
        int ipix, idet;
        T bound0;
        if (geom == DDO_ARC) {
            /* FanArcDisCPU2d.cpp:102-116 (x) and :172-186 (y) */
            T tan0, tan1;
            if (xb) {
                tan0 = ((vw->srcx - p0) == 0) ? (T)1e10 : vw->srcy / (vw->srcx - p0);
                tan1 = ((bin + view) == 0) ? (T)1e10 : (T)(-1 / tan((double)(bin + view)));
            } else {
                tan0 = (vw->srcy - p0) / vw->srcx;
                tan1 = (T)(-1 / tan((double)(bin + view)));
            }
            T delta = (T)atan((double)((tan0 - tan1) / (1 + tan0 * tan1)));
            idet = (int)floor(D / 2.0 + delta * (T)vw->flag / ds);
            if (idet < 0) {
                bound0 = vw->dp[0];
                ipix = (int)floor((double)((bound0 - p0) / pint));
                idet = 0;
            } else {
                bound0 = p0;
                ipix = 0;
            }
        } else {
            const T d0 = (geom == DDO_PARA) ? vw->det0 : vw->dp[0];
            bound0 = (T)fmax((double)p0, (double)d0);
            if (p0 == bound0) {
                ipix = 0;
                if (geom == DDO_PARA) {
                    idet = (int)floor((double)((bound0 - d0) / vw->di));
                } else {
                    /* FanFlatDisCPU2d.cpp:105-107 / :174-176 */
                    T back = xb ? vw->srcy * bound0 / ((bound0 - vw->srcx) * s / c + vw->srcy)
                                : vw->srcx * bound0 / ((bound0 - vw->srcy) * c / s + vw->srcx);
                    idet = (int)floor((double)((back - vw->det0xy) / vw->di));
                }
            } else {
                ipix = (int)floor((double)((bound0 - p0) / pint));
                idet = 0;
            }
        }
        if (idet < 0) idet = 0; /* the reference reads out of bounds here */
        if (ipix < 0) ipix = 0; /* likewise (a source inside the image); the kernels clamp too */

        T point1 = (T)(ipix + 1) * pint + p0;
        T det1 = 0;
        if (idet < D)
            det1 = (geom == DDO_PARA) ? (T)(idet + 1) * vw->di + vw->det0 : vw->dp[idet + 1];
        /* pixel centre for the FBP weight: FanFlatDisCPU2d.cpp:490, :565 */
        T pcx = xb ? (T)((ipix + 0.5) * sx + axis0) : lpos;
        T pcy = xb ? lpos : (T)((ipix + 0.5) * sy + axis0);

        while (ipix < npix && idet < D) {
            const int step_pix = (point1 < det1);
            const T seg = step_pix ? point1 - bound0 : det1 - bound0;
            T coef;
            if (geom != DDO_PARA && trans_scale) coef = seg * vw->bcoef[idet];
            else coef = seg * line_coef;
            const long long pix = xb ? (long long)line * W + ipix
                                     : (long long)(H - 1 - ipix) * W + line;
            const long long det = (long long)v * D + (vw->flip ? D - 1 - idet : idet);
            T wgt = 0;
            if (fbp)
                wgt = (geom == DDO_ARC) ? FN(cw_arc)(vw->srcx, vw->srcy, pcx, pcy)
                                        : FN(cw_flat)(vw->srcx, vw->srcy, pcx, pcy, R);
            FN(emit2)(op, in, out, batch, pix, pixstride, det, detstride, coef, wgt, fbp,
                      geom == DDO_ARC, atomic);
            if (step_pix) {
                bound0 = point1;
                ipix++;
                if (xb) pcx += sx; else pcy += sy;
                point1 += pint;
            } else {
                bound0 = det1;
                idet++;
                if (geom == DDO_PARA) det1 += vw->di;
                else if (idet < D) det1 = vw->dp[idet + 1];
            }
        }
    }
}

typedef struct {
    const ddo_geom2 *g;
    int geom, op, batch, nthreads, tid;
    const float *angles;
    const T *in;
    T *out;
} FN(job2);

static void *FN(thread2)(void *arg)
{
    FN(job2) *j = (FN(job2) *)arg;
    const ddo_geom2 *g = j->g;
    /* view split: ParaDisCPU2d.cpp:41-43 */
    const int per = (g->nv - 1) / j->nthreads + 1;
    const int v0 = per * j->tid;
    const int v1 = (v0 + per > g->nv) ? g->nv : v0 + per;
    FN(view2) vw;
    vw.dp = (T *)malloc(sizeof(T) * (g->nd + 1));
    vw.bcoef = (T *)malloc(sizeof(T) * (g->nd + 1));
    for (int v = v0; v < v1; v++) {
        const T view = (T)j->angles[v];
        FN(setup_view2)(g, j->geom, view, &vw);
        FN(walk_view2)(g, j->geom, j->op, v, view, &vw, j->in, j->out, j->batch,
                       j->nthreads > 1);
    }
    free(vw.dp);
    free(vw.bcoef);
    return NULL;
}

/* 2-D entry: `in`/`out` follow the reference layouts (image (B,H,W),
 * sinogram (B,V,D)); `out` must be zeroed by the caller (RadonTorch.cpp:41,
 * :68 zero the CPU outputs).  nthreads <= 0 picks the reference's own rule
 * min(ceil(V/128), cores) (ParaDisCPU2d.cpp:338-340). */
int FN(ddo_run2d)(const ddo_geom2 *g, int geom, int op, const float *angles,
                  const T *in, T *out, int batch, int nthreads)
{
    if (!g || g->width <= 0 || g->height <= 0 || g->nv <= 0 || g->nd <= 0 || batch <= 0)
        return -1;
    if (geom < DDO_PARA || geom > DDO_ARC || op < DDO_PROJ || op > DDO_BPROJ_TW) return -1;
    if (geom == DDO_PARA && (op == DDO_BPROJ_W || op == DDO_BPROJ_TW)) return -1;
    if (nthreads <= 0) nthreads = ddo_default_threads(g->nv);
    if (nthreads > g->nv) nthreads = g->nv;
    FN(job2) jobs[DDO_MAX_THREADS];
    pthread_t th[DDO_MAX_THREADS];
    if (nthreads > DDO_MAX_THREADS) nthreads = DDO_MAX_THREADS;
    for (int t = 0; t < nthreads; t++) {
        jobs[t].g = g; jobs[t].geom = geom; jobs[t].op = op; jobs[t].batch = batch;
        jobs[t].nthreads = nthreads; jobs[t].tid = t; jobs[t].angles = angles;
        jobs[t].in = in; jobs[t].out = out;
    }
    if (nthreads == 1) {
        FN(thread2)(&jobs[0]);
        return 0;
    }
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, FN(thread2), &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* 3-D (cone-flat, cone-arc, spiral): follows deeprecon/cuda/dis3d/<geom>DisCUDA3d.cu,     */
/* the reference has no CPU path for these (RadonTorch.cpp:604).             */
/* ------------------------------------------------------------------------ */

/* |c| / sqrt(a^2+b^2+c^2) evaluated in FP32 like the device function
 * ConeFlatDisCUDA3d.cu:21-23. */
static T FN(tricos3)(T a, T b, T c)
{
    return (T)fabs((double)c) / (T)sqrt((double)(a * a + b * b + c * c));
}

typedef struct {
    int xb, flip, flag;
    T s, c, view;
    T srcx, srcy, srcz;
    T colsz, colshift;     /* detector column pitch / shift (arc: radians)  */
    T sdd, iso;            /* (spiral-corrected) distances                  */
    T axial;               /* spiral: table axial source position          */
    T detcol0xy;           /* flat: x (y) of virtual column boundary 0      */
    T vds, vbs;            /* flat: virtual column pitch / shift            */
    T di;                  /* flat: column pitch projected on the axis      */
    T bp_scale;            /* DD-BP per-bin scale: VirDetColSize / DetColRad */
    T *dp;                 /* C+1 sorted column boundaries on the axis       */
    T *mag;                /* C per-column row magnification onto the plane  */
} FN(view3);

/* Per-view set-up: ConeFlatDisCUDA3d.cu:62-105 / :178-208,
 * ConeArcDisCUDA3d.cu:40-60 / :148-165, SpiralDisCUDA3d.cu:39-82. */
static void FN(setup_view3)(const ddo_geom3 *g, int geom, T view, const float *sp, int v,
                            FN(view3) *w)
{
    const int C = g->ncol;
    const T R = (T)g->iso_source, SDD = (T)g->source_detector;
    T dc = (T)g->col_size, cshift = (T)g->col_shift;
    T ang = view;
    w->view = view;
    w->di = 0;
    w->detcol0xy = 0;
    w->axial = 0;
    w->vds = w->vbs = 0;
    w->iso = R;
    w->sdd = SDD;
    w->srcz = 0;
    if (geom == DDO_SPIRAL) {
        const int nv = g->nv;
        const T axial = (T)sp[v], drad = (T)sp[nv + v], dang = (T)sp[2 * nv + v];
        const T daxial = (T)sp[3 * nv + v];
        w->iso = R + drad;
        w->sdd = SDD + drad;
        dc = (T)g->col_size * SDD / w->sdd;
        cshift = (T)g->col_shift * SDD / w->sdd - dang * (w->sdd - w->iso) / w->sdd;
        ang = view + dang;
        w->srcz = axial + daxial;
        w->axial = axial;
    }
    w->colsz = dc;
    w->colshift = cshift;
    w->s = (T)sin((double)ang);
    w->c = (T)cos((double)ang);
    const T s = w->s, c = w->c;
    {   /* branch from the FP32-rounded trig at every precision (see 2-D) */
        const float cf = (float)cos((double)ang), sf = (float)sin((double)ang);
        w->xb = (cf * cf > 0.5);
        w->flip = w->xb ? (cf < 0) : (sf < 0);
    }
    w->flag = w->flip ? -1 : 1;
    w->srcx = -s * w->iso;
    w->srcy = c * w->iso;
    if (geom == DDO_CONE_FLAT) {
        const T vds = R / SDD * dc, vbs = R / SDD * cshift;
        for (int k = 0; k <= C; k++) {
            double u = w->flip ? (C / 2.0 - k) * vds + vbs : (k - C / 2.0) * vds + vbs;
            T dx = (T)(u * c), dy = (T)(u * s);
            if (k == 0) w->detcol0xy = w->xb ? dx : dy;
            w->dp[k] = w->xb ? FN(map2x)(w->srcx, w->srcy, dx, dy)
                             : FN(map2y)(w->srcx, w->srcy, dx, dy);
        }
        for (int k = 0; k < C; k++) {
            double u = w->flip ? (C / 2.0 - k - 0.5) * vds + vbs : (k + 0.5 - C / 2.0) * vds + vbs;
            T cen = w->xb ? (T)(u * s) : (T)(u * c);
            w->mag[k] = w->xb ? w->srcy / (w->srcy - cen) : w->srcx / (w->srcx - cen);
        }
        w->di = vds * (T)fabs((double)(w->xb ? c : s));
        w->bp_scale = vds;
        w->vds = vds;
        w->vbs = vbs;
    } else {
        /* arc / spiral: ConeArcDisCUDA3d.cu:49-60 */
        for (int k = 0; k <= C; k++) {
            T a = (T)(w->flip ? (C / 2.0 - k) * dc + cshift + view : (k - C / 2.0) * dc + cshift + view);
            T t = (T)tan((double)a);
            w->dp[k] = w->xb ? w->srcx + w->srcy * t : w->srcy + w->srcx / t;
        }
        for (int k = 0; k < C; k++) {
            /* centre of column k from its upper boundary angle (ConeArc :51, :56) */
            T a1 = (T)(w->flip ? (C / 2.0 - k - 1) * dc + cshift + view
                               : (k + 1 - C / 2.0) * dc + cshift + view);
            double ac = w->flip ? (double)a1 + 0.5 * dc : (double)a1 - 0.5 * dc;
            T cen = w->xb ? (T)(-cos(ac) * w->sdd + w->srcy) : (T)(sin(ac) * w->sdd + w->srcx);
            w->mag[k] = w->xb ? w->srcy / (w->srcy - cen) : w->srcx / (w->srcx - cen);
        }
        w->bp_scale = w->iso * dc;
    }
}

/* Walk one (view, detector row) pair over every image line: the per-thread
 * loop of ConeFlatDisCUDA3d.cu:106-170 (FP), :370-431 (ProjTrans),
 * :622-690 (BackProj), :875-945 (BackProjTrans) and the y-branch copies,
 * with the 256-column chunking removed (it does not change the segments). */
static void FN(walk_row3)(const ddo_geom3 *g, int geom, int op, int v, int r,
                          const FN(view3) *w, const T *in, T *out, int batch,
                          T *binacc, T *rp0, T *rp1, T *scale, int atomic)
{
    const int W = g->width, H = g->height, Dp = g->depth, C = g->ncol, Rn = g->nrow;
    const int V = g->nv;
    const T sx = (T)g->pix_x, sy = (T)g->pix_y, sz = (T)g->pix_z;
    const T pxs = (T)g->pix_xshift, pys = (T)g->pix_yshift;
    const T pzs = (geom == DDO_SPIRAL) ? (T)0 : (T)g->pix_zshift;
    const int xb = w->xb;
    const int nline = xb ? H : W, npix = xb ? W : H;
    const int fbp = (op == DDO_BPROJ_W || op == DDO_BPROJ_TW);
    const int proj_type = (op == DDO_PROJ || op == DDO_BPROJ_T || op == DDO_BPROJ_TW);
    const long long vox_b = (long long)W * H * Dp, det_b = (long long)V * Rn * C;

    /* row boundaries of detector row r (ConeFlat :68-69, ConeArc :40-41,
     * Spiral :49) */
    T row0z, row1z;
    if (geom == DDO_CONE_FLAT) {
        const T R = (T)g->iso_source, SDD = (T)g->source_detector;
        row0z = (T)((((double)r - Rn / 2.0) * (T)g->row_size + (T)g->row_shift) * R / SDD);
        row1z = row0z + R / SDD * (T)g->row_size;
    } else if (geom == DDO_CONE_ARC) {
        row0z = (T)(((double)r - Rn / 2.0) * (T)g->row_size + (T)g->row_shift);
        row1z = row0z + (T)g->row_size;
    } else {
        row0z = (T)(((double)r - Rn / 2.0) * (T)g->row_size + (double)w->axial +
                    (T)g->row_shift);
        row1z = row0z + (T)g->row_size;
    }
    /* per-column row boundaries on the plane and bin scales */
    const T pixl = xb ? sy : sx;
    for (int k = 0; k < C; k++) {
        if (geom == DDO_CONE_FLAT || geom == DDO_CONE_ARC) {
            rp0[k] = w->mag[k] * row0z;
            rp1[k] = w->mag[k] * row1z;
        } else {
            rp0[k] = w->mag[k] * (row0z - w->srcz) + w->srcz;
            rp1[k] = w->mag[k] * (row1z - w->srcz) + w->srcz;
        }
        const T coef1 = (w->dp[k + 1] - w->dp[k]) * (rp1[k] - rp0[k]);
        const T a = (T)((w->dp[k + 1] + w->dp[k]) / 2.0 - (xb ? w->srcx : w->srcy));
        const T b = (T)((rp1[k] + rp0[k]) / 2.0);
        const T coef2 = FN(tricos3)(a, b, xb ? w->srcy : w->srcx);
        scale[k] = (op == DDO_PROJ || op == DDO_PROJ_T) ? pixl / (coef1 * coef2) : w->bp_scale;
    }
    if (proj_type)
        for (int k = 0; k < batch * C; k++) binacc[k] = 0;

    const T axis0 = xb ? (T)(-W / 2.0 * sx + pxs) : (T)(-H / 2.0 * sy + pys);
    const T axis1 = xb ? (T)(W / 2.0 * sx + pxs) : (T)(H / 2.0 * sy + pys);
    const T z0 = (T)(-Dp / 2.0 * sz + pzs), z1 = (T)(Dp / 2.0 * sz + pzs);

    for (int line = 0; line < nline; line++) {
        const T lpos = xb ? (T)((H / 2.0 - line - 0.5) * sy + pys)
                          : (T)((line - W / 2.0 + 0.5) * sx + pxs);
        T p0, p1, p0z, p1z;
        if (xb) {
            p0 = FN(map2x)(w->srcx, w->srcy, axis0, lpos);
            p1 = FN(map2x)(w->srcx, w->srcy, axis1, lpos);
        } else {
            p0 = FN(map2y)(w->srcx, w->srcy, lpos, axis0);
            p1 = FN(map2y)(w->srcx, w->srcy, lpos, axis1);
        }
        const T m = xb ? w->srcy / (w->srcy - lpos) : w->srcx / (w->srcx - lpos);
        if (geom == DDO_SPIRAL) {
            p0z = m * (z0 - w->srcz) + w->srcz;
            p1z = m * (z1 - w->srcz) + w->srcz;
        } else {
            p0z = m * z0;
            p1z = m * z1;
        }
        const T pint = (p1 - p0) / (T)npix;
        const T pintz = (p1z - p0z) / (T)Dp;
        const T parea = pint * pintz;
        /* the reference walks each block of 256 detector columns separately
         * (ConeFlatDisCUDA3d.cu:53-56, :116-130): every block restarts the
         * walk, and with it the FP32 accumulation of the pixel boundaries */
        for (int c0 = 0; c0 < C; c0 += 256) {
        const int maxn = (C - c0 < 256) ? C - c0 : 256;
        int ipix, idet;
        T bound0;
        if (geom == DDO_CONE_FLAT) {
            bound0 = p0 > w->dp[c0] ? p0 : w->dp[c0];
            if (p0 == bound0) {
                T back = xb ? w->srcy * bound0 / ((bound0 - w->srcx) * w->s / w->c + w->srcy)
                            : w->srcx * bound0 / ((bound0 - w->srcy) * w->c / w->s + w->srcx);
                const double uc = w->flip ? (C / 2.0 - c0) * w->vds + w->vbs : (c0 - C / 2.0) * w->vds + w->vbs;
                const T col0 = xb ? (T)(uc * (double)w->c) : (T)(uc * (double)w->s);
                ipix = 0;
                idet = (int)floor((double)((back - col0) / w->di));
            } else {
                ipix = (int)floor((double)((bound0 - p0) / pint));
                idet = 0;
            }
        } else {
            /* ConeArcDisCUDA3d.cu:84-96, Spiral :93-105 */
            T tan0, tan1;
            const T base = w->colshift + w->view;
            if (xb) {
                tan0 = ((w->srcx - p0) == 0) ? (T)1e10 : w->srcy / (w->srcx - p0);
                tan1 = (base == 0) ? (T)1e10 : -1 / (T)tan((double)base);
            } else {
                tan0 = (w->srcy - p0) / w->srcx;
                tan1 = -1 / (T)tan((double)base);
            }
            T delta = (T)atan((double)((tan0 - tan1) / (1 + tan0 * tan1)));
            idet = (int)floor(C / 2.0 - c0 + delta * (T)w->flag / w->colsz);
            if (idet < 0) {
                bound0 = w->dp[c0];
                ipix = (int)floor((double)((bound0 - p0) / pint));
                idet = 0;
            } else {
                bound0 = p0;
                ipix = 0;
            }
        }
        if (idet < 0) idet = 0;
        T point1 = (T)(ipix + 1) * pint + p0;
        T det1 = (idet < maxn) ? w->dp[c0 + idet + 1] : 0;
        T pcx = xb ? (T)((ipix + 0.5) * sx + axis0) : lpos;
        T pcy = xb ? lpos : (T)((ipix + 0.5) * sy + axis0);
        while (ipix < npix && idet < maxn) {
            const int col = c0 + idet;
            T bz0 = p0z > rp0[col] ? p0z : rp0[col];
            const T bz1 = p1z < rp1[col] ? p1z : rp1[col];
            int islice = (bz0 == p0z) ? 0 : (int)floor((double)((bz0 - p0z) / pintz));
            T pz1 = (T)(islice + 1) * pintz + p0z;
            const int step_pix = (point1 < det1);
            T coef = step_pix ? point1 - bound0 : det1 - bound0;
            if (op != DDO_PROJ && op != DDO_PROJ_T) {
                coef = coef / parea;
                if (fbp) {
                    if (geom == DDO_CONE_FLAT) coef *= FN(cw_flat)(w->srcx, w->srcy, pcx, pcy, w->iso);
                    else coef /= FN(cw_arc)(w->srcx, w->srcy, pcx, pcy);
                }
            }
            const int lrow = xb ? line : H - 1 - ipix;
            const int lcol = xb ? ipix : line;
            const long long detidx = ((long long)v * Rn + r) * C + (w->flip ? C - 1 - col : col);
            while (bz0 < bz1 && islice < Dp) {
                pz1 = (pz1 > bz1) ? bz1 : pz1;
                const long long vox = ((long long)islice * H + lrow) * W + lcol;
                const T zc = (pz1 - bz0) * coef;
                for (int b = 0; b < batch; b++) {
                    if (proj_type) {
                        binacc[b * C + col] += zc * in[b * vox_b + vox];
                    } else {
                        const T val = zc * (in[b * det_b + detidx] * scale[col]);
                        if (atomic) FN(atomic_add)(out + b * vox_b + vox, val);
                        else out[b * vox_b + vox] += val;
                    }
                }
                bz0 = pz1;
                islice++;
                pz1 += pintz;
            }
            if (step_pix) {
                bound0 = point1;
                ipix++;
                if (xb) pcx += sx; else pcy += sy;
                point1 += pint;
            } else {
                bound0 = det1;
                idet++;
                if (idet < maxn) det1 = w->dp[c0 + idet + 1];
            }
        }
        }
    }
    if (proj_type) {
        for (int b = 0; b < batch; b++)
            for (int k = 0; k < C; k++) {
                const long long detidx = ((long long)v * Rn + r) * C + (w->flip ? C - 1 - k : k);
                out[b * det_b + detidx] = binacc[b * C + k] * scale[k];
            }
    }
}

typedef struct {
    const ddo_geom3 *g;
    int geom, op, batch, nthreads, tid;
    const float *angles, *sp;
    const T *in;
    T *out;
} FN(job3);

static void *FN(thread3)(void *arg)
{
    FN(job3) *j = (FN(job3) *)arg;
    const ddo_geom3 *g = j->g;
    const int per = (g->nv - 1) / j->nthreads + 1;
    const int v0 = per * j->tid;
    const int v1 = (v0 + per > g->nv) ? g->nv : v0 + per;
    FN(view3) w;
    const int C = g->ncol;
    w.dp = (T *)malloc(sizeof(T) * (C + 1));
    w.mag = (T *)malloc(sizeof(T) * (C + 1));
    T *scratch = (T *)malloc(sizeof(T) * ((size_t)j->batch * C + 3 * (size_t)C + 4));
    T *rp0 = scratch, *rp1 = scratch + C, *scale = scratch + 2 * (size_t)C;
    T *bin = scratch + 3 * (size_t)C;
    for (int v = v0; v < v1; v++) {
        const T view = (T)j->angles[v];
        FN(setup_view3)(g, j->geom, view, j->sp, v, &w);
        for (int r = 0; r < g->nrow; r++)
            FN(walk_row3)(g, j->geom, j->op, v, r, &w, j->in, j->out, j->batch, bin, rp0,
                          rp1, scale, j->nthreads > 1);
    }
    free(w.dp);
    free(w.mag);
    free(scratch);
    return NULL;
}

int FN(ddo_run3d)(const ddo_geom3 *g, int geom, int op, const float *angles,
                  const float *sp, const T *in, T *out, int batch, int nthreads)
{
    if (!g || g->width <= 0 || g->height <= 0 || g->depth <= 0 || g->nv <= 0 ||
        g->ncol <= 0 || g->nrow <= 0 || batch <= 0)
        return -1;
    if (geom < DDO_CONE_FLAT || geom > DDO_SPIRAL || op < DDO_PROJ || op > DDO_BPROJ_TW) return -1;
    if (geom == DDO_SPIRAL && !sp) return -1;
    if (nthreads <= 0) nthreads = ddo_default_threads(g->nv);
    if (nthreads > g->nv) nthreads = g->nv;
    if (nthreads > DDO_MAX_THREADS) nthreads = DDO_MAX_THREADS;
    FN(job3) jobs[DDO_MAX_THREADS];
    pthread_t th[DDO_MAX_THREADS];
    for (int t = 0; t < nthreads; t++) {
        jobs[t].g = g; jobs[t].geom = geom; jobs[t].op = op; jobs[t].batch = batch;
        jobs[t].nthreads = nthreads; jobs[t].tid = t; jobs[t].angles = angles;
        jobs[t].sp = sp; jobs[t].in = in; jobs[t].out = out;
    }
    if (nthreads == 1) {
        FN(thread3)(&jobs[0]);
        return 0;
    }
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, FN(thread3), &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Start-index scan of deeprecon's CUDA kernels                             */
/* ------------------------------------------------------------------------ */

/* deeprecon's CUDA kernels start the walk of each (view, block of 256
 * detector columns, image line) at a detector index and a pixel index taken
 * from two different formulas: the flat-detector kernels map the line's first
 * pixel boundary back onto the detector (FanFlatDisCUDA2d.cu:96-104,
 * ConeFlatDisCUDA3d.cu:116-127), the arc ones compare angles through atan
 * and then locate the block's first column among the pixels
 * (FanArcDisCUDA2d.cu:97-110, ConeArcDisCUDA3d.cu:84-96, SpiralDisCUDA3d.cu:93-105).
 * Both are >= 0 in exact arithmetic, but where the image edge and the
 * block's first column boundary coincide to within rounding one of them can
 * floor to -1, and the kernel then indexes shared memory (ProjTemp[-1]) or
 * its output (atomicAdd at column -1) out of bounds.  The scan evaluates
 * those start values for every (view, block, line) with the reference's FP32
 * arithmetic and counts the starts that lie within `margin` (in detector
 * cells or pixels; ten times that for the arc kernels' angle-based detector
 * index, whose atan/tan chain rounds more loosely) of such a rounding,
 * taking either branch of a start decision whose two operands tie to within
 * 2e-6 relative (17 to 33 FP32 ulps: the device code's fused multiply-adds
 * and its own tan/atan move them by a few).  `per_view` (optional, nv
 * entries) receives the count of each view, so that a case can be run on the
 * views without any.  A case with count 0 can be given to
 * the reference kernels; one with a non-zero count is not run there.  The
 * parallel beam needs no scan: its start is the difference of the two values
 * compared (ParaDisCUDA2d.cu:56-62), which is >= 0 in any rounding. */

static int FN(flat_start_hazard)(int xb, T p0, T pint, T dpc0, T s, T c, T srcx, T srcy,
                                 double u0, T di, double margin)
{
    const double tie = 2e-6 * fmax(fabs((double)p0), fabs((double)dpc0));
    (void)pint;
    if (!(p0 >= dpc0 || fabs((double)(p0 - dpc0)) <= tie)) return 0;
    const T back = xb ? srcy * p0 / ((p0 - srcx) * s / c + srcy)
                      : srcx * p0 / ((p0 - srcy) * c / s + srcx);
    const T col0 = xb ? (T)(u0 * (double)c) : (T)(u0 * (double)s);
    return ((double)((back - col0) / di) < margin);
}

static int FN(arc_start_hazard)(int xb, T p0, T pint, T dpc0, T srcx, T srcy, T base,
                                double det_half_minus_c0, int flag, T colsz, double margin)
{
    T tan0, tan1;
    if (xb) {
        tan0 = ((srcx - p0) == 0) ? (T)1e10 : srcy / (srcx - p0);
        tan1 = (base == 0) ? (T)1e10 : (T)(-1 / tan((double)base));
    } else {
        tan0 = (srcy - p0) / srcx;
        tan1 = (T)(-1 / tan((double)base));
    }
    const T delta = (T)atan((double)((tan0 - tan1) / (1 + tan0 * tan1)));
    const double v = det_half_minus_c0 + (double)(delta * (T)flag / colsz);
    if (v >= 10 * margin) return 0;
    return ((double)((dpc0 - p0) / pint) < margin);
}

long long FN(ddo_scan2d)(const ddo_geom2 *g, int geom, const float *angles, double margin,
                         int *per_view)
{
    if (per_view)
        for (int v = 0; v < g->nv; v++) per_view[v] = 0;
    if (geom == DDO_PARA) return 0;
    const int W = g->width, H = g->height, D = g->nd;
    const T sx = (T)g->pix_x, sy = (T)g->pix_y, ds = (T)g->det_size;
    const T R = (T)g->iso_source, SDD = (T)g->source_detector;
    const T pxs = (T)g->pix_xshift, pys = (T)g->pix_yshift, bin = (T)g->bin_shift;
    const T vds = R / SDD * ds, vbs = R / SDD * bin;
    FN(view2) vw;
    vw.dp = (T *)malloc(sizeof(T) * (D + 1));
    vw.bcoef = (T *)malloc(sizeof(T) * (D + 1));
    long long count = 0;
    for (int v = 0; v < g->nv; v++) {
        const T view = (T)angles[v];
        FN(setup_view2)(g, geom, view, &vw);
        const int xb = vw.xb, nline = xb ? H : W, npix = xb ? W : H;
        const T axis0 = xb ? (T)(-W / 2.0 * sx + pxs) : (T)(-H / 2.0 * sy + pys);
        const T axis1 = xb ? (T)(W / 2.0 * sx + pxs) : (T)(H / 2.0 * sy + pys);
        for (int line = 0; line < nline; line++) {
            const T lpos = xb ? (T)((H / 2.0 - line - 0.5) * sy + pys)
                              : (T)((line - W / 2.0 + 0.5) * sx + pxs);
            const T p0 = xb ? FN(map2x)(vw.srcx, vw.srcy, axis0, lpos)
                            : FN(map2y)(vw.srcx, vw.srcy, lpos, axis0);
            const T p1 = xb ? FN(map2x)(vw.srcx, vw.srcy, axis1, lpos)
                            : FN(map2y)(vw.srcx, vw.srcy, lpos, axis1);
            const T pint = (p1 - p0) / (T)npix;
            for (int c0 = 0; c0 < D; c0 += 256) {
                int hz;
                if (geom == DDO_FLAT) {
                    const double u0 = vw.flip ? (D / 2.0 - c0) * vds + vbs : (c0 - D / 2.0) * vds + vbs;
                    hz = FN(flat_start_hazard)(xb, p0, pint, vw.dp[c0], vw.s, vw.c, vw.srcx,
                                               vw.srcy, u0, vw.di, margin);
                } else {
                    hz = FN(arc_start_hazard)(xb, p0, pint, vw.dp[c0], vw.srcx, vw.srcy,
                                              bin + view, D / 2.0 - c0, vw.flag, ds, margin);
                }
                count += hz;
                if (per_view) per_view[v] += hz;
            }
        }
    }
    free(vw.dp);
    free(vw.bcoef);
    return count;
}

long long FN(ddo_scan3d)(const ddo_geom3 *g, int geom, const float *angles, const float *sp,
                         double margin, int *per_view)
{
    if (geom == DDO_SPIRAL && !sp) return -1;
    if (per_view)
        for (int v = 0; v < g->nv; v++) per_view[v] = 0;
    const int W = g->width, H = g->height, C = g->ncol;
    const T sx = (T)g->pix_x, sy = (T)g->pix_y;
    const T pxs = (T)g->pix_xshift, pys = (T)g->pix_yshift;
    FN(view3) w;
    w.dp = (T *)malloc(sizeof(T) * (C + 1));
    w.mag = (T *)malloc(sizeof(T) * (C + 1));
    long long count = 0;
    for (int v = 0; v < g->nv; v++) {
        const T view = (T)angles[v];
        FN(setup_view3)(g, geom, view, sp, v, &w);
        const int xb = w.xb, nline = xb ? H : W, npix = xb ? W : H;
        const T axis0 = xb ? (T)(-W / 2.0 * sx + pxs) : (T)(-H / 2.0 * sy + pys);
        const T axis1 = xb ? (T)(W / 2.0 * sx + pxs) : (T)(H / 2.0 * sy + pys);
        for (int line = 0; line < nline; line++) {
            const T lpos = xb ? (T)((H / 2.0 - line - 0.5) * sy + pys)
                              : (T)((line - W / 2.0 + 0.5) * sx + pxs);
            const T p0 = xb ? FN(map2x)(w.srcx, w.srcy, axis0, lpos)
                            : FN(map2y)(w.srcx, w.srcy, lpos, axis0);
            const T p1 = xb ? FN(map2x)(w.srcx, w.srcy, axis1, lpos)
                            : FN(map2y)(w.srcx, w.srcy, lpos, axis1);
            const T pint = (p1 - p0) / (T)npix;
            for (int c0 = 0; c0 < C; c0 += 256) {
                int hz;
                if (geom == DDO_CONE_FLAT) {
                    const double u0 = w.flip ? (C / 2.0 - c0) * w.vds + w.vbs
                                             : (c0 - C / 2.0) * w.vds + w.vbs;
                    hz = FN(flat_start_hazard)(xb, p0, pint, w.dp[c0], w.s, w.c, w.srcx,
                                               w.srcy, u0, w.di, margin);
                } else {
                    hz = FN(arc_start_hazard)(xb, p0, pint, w.dp[c0], w.srcx, w.srcy,
                                              w.colshift + w.view, C / 2.0 - c0, w.flag,
                                              w.colsz, margin);
                }
                count += hz;
                if (per_view) per_view[v] += hz;
            }
        }
    }
    free(w.dp);
    free(w.mag);
    return count;
}
