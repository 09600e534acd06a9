// Shared device code of the 2-D DD projector: layouts, the integral-form
// evaluation and the two work-item bodies (forward = detector gathers,
// adjoint = pixel gathers).  Included by dd2d.cu (single-geometry launches)
// and dd2d_batch.cu (persistent launches over uneven instances).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cooperative_groups.h>

#include "../../include/pridediff_dd.h"
#include "dd_geom2d.cuh"
#include "dd_tma.cuh"

namespace dd2 {


constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kBinsPerWarp = 31;   // 32 boundaries -> 31 bins per warp pass
constexpr int kBI = 4;             // images per CTA (geometry amortised over them)
constexpr int kTile = 32;          // adjoint work item: 32 x 32 pixels
// Adjoint-map entries per walked line of a tile: the boundaries of a 32-pixel
// run plus one below it, from an even first entry (36), padded to an odd
// number of 8-byte entries so that the lanes of a warp reading 32 different
// lines' rows hit distinct shared-memory banks.
constexpr int kMapE = 37;
// One adjoint-map block (a view, a tile): kTile rows of kMapE entries {bin,
// offset}, then the kTile lines' DD-BP scales; one bulk copy moves it.
constexpr int kMapBlkBytes = kTile * kMapE * 8 + kTile * 4;

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
__host__ __device__ inline int rs_entries(int n) { return (n + 2) & ~1; }   // n+1 float2, 16-B rows

// ---------------------------------------------------------------------------
// Workspace layout
// ---------------------------------------------------------------------------
struct PlanLayout {
    size_t views, ang, dp, bcoef, lines, dlines, axisv, amap, trange, total;
    int nl;   // line records per view = max(H, W)
};

// Adjoint map of fan beams, one block per (view, tile) in tile-major order.
// Entry e of a walked line holds its boundary e - 1 (e in 0 .. map_stride()-1
// over the line); a block keeps, for each of the tile's kTile walked lines,
// the kMapE entries from the tile's first entry (map_first()).
__host__ __device__ inline int map_stride(const dd_geom2d *g) {
    return rs_entries(g->width > g->height ? g->width : g->height);
}
// 32 x 32 tiles of the image (the adjoint's work items); tile = ty * ntx + tx
__host__ __device__ inline int tiles_x(const dd_geom2d *g) { return (g->width + 31) / 32; }
__host__ __device__ inline int tiles_n(const dd_geom2d *g) { return tiles_x(g) * ((g->height + 31) / 32); }
// First map entry a tile's block keeps.  Rows (xb views): pixels c0 .. c0+31
// have boundaries c0-1 .. c0+31, entries c0 .. c0+32.  Columns: pixels
// H-r0-32 .. H-r0-1 along the column, entries from an even index at or below
// H-r0-32 (so that 36 entries always reach H-r0).
__host__ __device__ inline int map_first(const dd_geom2d *g, int xb, int c0, int r0) {
    if (xb) return c0;
    const int lo = g->height - r0 - kTile;
    return (lo > 0 ? lo : 0) & ~1;
}

// with_map = false leaves out the adjoint map (plans that only serve the
// forward-type operators, e.g. one-shot forward calls); every other offset is
// the same either way.
inline PlanLayout plan_layout(int scan, const dd_geom2d *g, int V, bool with_map = true) {
    PlanLayout L;
    const int D = g->num_det;
    L.nl = g->height > g->width ? g->height : g->width;
    size_t o = 0;
    L.views = o; o = align_up(o + sizeof(DdView2) * (size_t)V, 256);
    L.ang = o; o = align_up(o + sizeof(float) * (size_t)V, 256);
    L.dp = o; o = align_up(o + sizeof(float) * (size_t)V * (D + 1), 256);
    L.bcoef = o; o = align_up(o + sizeof(float) * (size_t)V * (D + 1), 256);
    L.lines = o; o = align_up(o + sizeof(DdLine) * (size_t)V * L.nl, 256);
    L.dlines = o;
    if (scan == DD_SCAN_PARA) o = align_up(o + sizeof(DdLine) * (size_t)V * L.nl, 256);
    // parallel beam: the views that walk rows and those that walk columns
    // ({count rows, count columns, rows' views[V], columns' views[V]})
    L.axisv = o;
    if (scan == DD_SCAN_PARA) o = align_up(o + sizeof(int) * (2 * (size_t)V + 2), 256);
    L.amap = L.trange = o;
    if (scan != DD_SCAN_PARA && with_map) {
        L.amap = o; o = align_up(o + (size_t)kMapBlkBytes * V * tiles_n(g), 256);
        L.trange = o; o = align_up(o + sizeof(int2) * (size_t)V * tiles_n(g), 256);
    }
    L.total = o;
    return L;
}

struct ApplyLayout {
    size_t tabx, taby, dtab, status, total;
};

inline bool op_is_forward(int op) {
    return op == DD_OP_PROJ || op == DD_OP_BPROJ_T || op == DD_OP_BPROJ_TW;
}

inline ApplyLayout apply_layout(int op, const dd_geom2d *g, int B, int V) {
    ApplyLayout L;
    size_t o = 0;
    L.tabx = L.taby = L.dtab = 0;
    if (op_is_forward(op)) {
        L.tabx = o; o = align_up(o + sizeof(float2) * (size_t)B * g->height * rs_entries(g->width), 256);
        L.taby = o; o = align_up(o + sizeof(float2) * (size_t)B * g->width * rs_entries(g->height), 256);
    } else {
        L.dtab = o; o = align_up(o + sizeof(float2) * (size_t)B * V * rs_entries(g->num_det), 256);
    }
    L.status = o; o = align_up(o + 256, 256);
    L.total = o;
    return L;
}

// ---------------------------------------------------------------------------
// Shared device pieces of the integral evaluation
// ---------------------------------------------------------------------------
// Per-piece constants K_p of one line for table `tab` (lane p < npiece).
// F(u) = K_p + dl_p S_j + r x_j on piece p (see file header).
__device__ __forceinline__ float piece_K(const DdLine &L, const float2 *tab, int lane) {
    const int np = L.h.npiece;
    float term = 0.0f;
    if (lane < np) {
        const DdPiece P = L.p[lane];
        const int first = (lane == 0) ? L.h.i0 : L.p[lane - 1].gb + 1;
        const float fv = FADD(P.Q, FMUL((float)(first - P.gb), P.dl));
        const float prevQ = (lane == 0) ? L.h.bound0 : L.p[lane - 1].Q;
        const float prevdl = (lane == 0) ? 0.0f : L.p[lane - 1].dl;
        const float2 e0 = tab[first];
        const float S1 = tab[first + 1].x;
        term = fmaf(prevdl, e0.x, fmaf(e0.y, fv - prevQ, -P.dl * S1));
    }
    for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, term, o);
        if (lane >= o) term += y;
    }
    return term;
}

// FBP-weight pixel centre a * pitch + shift, a an exact half-integer offset:
// one FMA rounds the exact value once.  The reference evaluates the same
// expression in FP64 and rounds that to FP32, which gives the same float
// unless the exact value lies within 2^-53 (relative) of an FP32 rounding
// boundary -- and FP64 arithmetic runs at a small fraction of the FP32 rate.
__device__ __forceinline__ float pix_centre(float a, float pitch, float shift) { return fmaf(a, pitch, shift); }

// ---------------------------------------------------------------------------
// Prefix tables in double-float arithmetic.  A sum is carried as an unevaluated
// pair hi + lo of floats (two-sum and FMA two-product are exact), about 48
// significant bits; hi of the pair is the sum rounded to FP32.  FP64 would do
// the same, but GB300 runs FP64 at a small fraction of its FP32 rate and the
// tables' scans were bound by it.
// ---------------------------------------------------------------------------
struct DdF {
    float hi, lo;
};
__device__ __forceinline__ DdF df_add(DdF a, DdF b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    const float t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, t);
    return {hi, __fsub_rn(t, __fsub_rn(hi, s))};
}
__device__ __forceinline__ DdF df_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ DdF df_shfl_up(DdF a, int o) {
    return {__shfl_up_sync(0xffffffffu, a.hi, o), __shfl_up_sync(0xffffffffu, a.lo, o)};
}
__device__ __forceinline__ DdF df_shfl(DdF a, int l) {
    return {__shfl_sync(0xffffffffu, a.hi, l), __shfl_sync(0xffffffffu, a.lo, l)};
}

// One warp: entries k = 0 .. n of t get (sum_{m<k} v_m, x_k) for the values
// v_k = x_k * w_k produced by val(k, &x, &w) (x = w = 0 past the end).
template <typename F>
__device__ __forceinline__ void warp_prefix_table(int n, float2 *t, int lane, F val) {
    DdF run = {0.0f, 0.0f};
    for (int k0 = 0; k0 <= n; k0 += 32) {
        const int k = k0 + lane;
        float x = 0.0f, w = 0.0f;
        if (k < n) val(k, &x, &w);
        DdF inc = df_prod(x, w);
        for (int o = 1; o < 32; o <<= 1) {
            const DdF y = df_shfl_up(inc, o);
            if (lane >= o) inc = df_add(inc, y);
        }
        DdF prev = df_shfl_up(inc, 1);
        if (lane == 0) prev = {0.0f, 0.0f};
        if (k <= n) t[k] = make_float2(df_add(run, prev).hi, x);
        run = df_add(run, df_shfl(inc, 31));
    }
}

// FBP weight of a fan-beam pixel centre (px, py) for the source (sx, sy):
// flat detector r^2 / (r - s.p / r)^2 (FanFlatDisCPU2d.cpp:693, r the
// source radius), evaluated as (r^2 / (r^2 - s.p))^2 with one fast division
// (__fdividef: within 2 ulp for these magnitudes) instead of two IEEE
// divisions; arc detector 1 / |s - p|^2 (FanArcDisCPU2d.cpp:703).  Within a
// few ulp of the reference's FP32 sequence; the forward-type and the
// adjoint-type kernels both use it, so BackProjWeighted and
// BackProjTransWeighted stay exact transposes.
template <int GEOM>
__device__ __forceinline__ float fan_fbp_weight(float sx, float sy, float px, float py, float r) {
    if (GEOM == DD_GEOM_ARC) {
        const float a = sx - px, b = sy - py;
        return __fdividef(1.0f, fmaf(a, a, b * b));
    }
    const float r2 = r * r;
    const float t = __fdividef(r2, r2 - fmaf(sx, px, sy * py));
    return t * t;
}

struct Loc {
    int p, j;
    float dl, r;
};

__device__ __forceinline__ Loc locate(const DdLine &L, float u) {
    Loc l;
    float rr;
    dd_locate(&L, u, &l.p, &l.j, &rr);
    l.r = rr;
    l.dl = L.p[l.p].dl;
    return l;
}

// ---------------------------------------------------------------------------
// Forward-type kernel (Proj, BackProjTrans, BackProjTransWeighted): detector
// gathers.  CTA = (view, group of kBI images); loops over the view's walked
// lines with the line record and the kBI line tables double-buffered in
// shared memory by TMA bulk copies.
// ---------------------------------------------------------------------------
// Detector passes of a 256-thread CTA (8 warps x 31 bins each) rounded up to
// the instantiated classes; NPASS sizes the per-thread accumulators, so a
// smaller class means fewer registers and more resident CTAs per SM.
__host__ __device__ inline int npass_class(int D, int nw = kWarps) {
    const int n = (D + nw * kBinsPerWarp - 1) / (nw * kBinsPerWarp);
    return n <= 1 ? 1 : n <= 2 ? 2 : n <= 3 ? 3 : n <= 4 ? 4 : 8;
}

struct FwdSmem {
    // dynamic layout offsets (bytes)
    int rec, drec, tab, kt, dp, bar, total;
};

// Forward CTAs per work item: a cluster of kFwdCluster CTAs shares a view's
// lines (rank r walks lines r, r + kFwdCluster, ...), so items are shorter and
// the last ones leave fewer SMs idle; rank 0 adds the others' sums through
// distributed shared memory.
constexpr int kFwdCluster = 2;

// (BackProjTransWeighted uses the same layout: its weights live in registers.)
// cl > 1: the line tables' space also holds a CTA's sums for the combine
// (npass_class(D) passes x bi images x 32 lanes x nw warps floats).
__host__ __device__ inline FwdSmem fwd_smem(int geom, int D, int rsmax, int bi = kBI, int cl = 1,
                                            int nw = kWarps) {
    FwdSmem s;
    int o = 0;
    s.rec = o; o += 2 * (int)sizeof(DdLine);
    s.drec = o; if (geom == DD_GEOM_PARA) o += 2 * (int)sizeof(DdLine);
    s.tab = o;
    {
        const int tabs = 2 * bi * rsmax * (int)sizeof(float2);
        const int red = cl > 1 ? npass_class(D, nw) * bi * nw * 32 * (int)sizeof(float) : 0;
        o += tabs > red ? tabs : red;
    }
    s.kt = o; o += bi * 32 * (int)sizeof(float);   // K of the pixel pieces
    s.dp = o; o += ((D + 1 + 3) & ~3) * (int)sizeof(float);
    s.bar = o; o += 2 * (int)sizeof(uint64_t);
    s.total = (o + 127) & ~127;
    return s;
}

// One forward work item: a view of one instance and a group of <= kBI of its
// images.  Epilogue: out = beta * acc (sub == nullptr) or beta * acc - sub
// (data-consistency residual A x - y, written without a separate pass).
struct FwdItem {
    int v, b0, nb, V, nl;
    const DdView2 *views;
    const float *dp, *bcoef;
    const DdLine *lines, *dlines;
    const float2 *tabx, *taby;   // prefix tables of image 0 of the instance
    float *out;                  // sinogram of image 0 of the instance
    const float *sub;            // optional, same layout as out
};

// Forward (detector-gather) evaluation of one work item.  The caller has
// initialised bar[0..1]; `ph` tracks the barriers' phases so that a
// persistent CTA can run many items back to back.  Returns false if a
// bounded wait timed out (copies in flight have been drained).
// CL > 1: the CTAs of a cluster of CL run the item together, rank r walking
// lines r, r + CL, ...; every rank returns after the combine, and all of them
// return false if any rank timed out.
template <int GEOM, int WEIGHTED, int NPASS, int BI = kBI, int NW = kWarps, int CL = 1>
__device__ bool fwd_view(const dd_geom2d &g, int op, const FwdItem &it, unsigned char *smem,
                         int Dmax, int rsmax, DdPhases &ph) {
    const int v = it.v, b0 = it.b0, nb = it.nb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rank = CL > 1 ? (int)cooperative_groups::this_cluster().block_rank() : 0;
    const int D = g.num_det;
    const DdView2 vw = it.views[v];
    const int xb = vw.xb;
    const int nline = xb ? g.height : g.width;
    const int npix = xb ? g.width : g.height;
    const int rs = rs_entries(npix);
    const FwdSmem L = fwd_smem(GEOM, Dmax, rsmax, BI, CL, NW);
    DdLine *rec = reinterpret_cast<DdLine *>(smem + L.rec);
    DdLine *drec = reinterpret_cast<DdLine *>(smem + L.drec);
    float2 *tab = reinterpret_cast<float2 *>(smem + L.tab);
    float *kt = reinterpret_cast<float *>(smem + L.kt);
    float *dps = reinterpret_cast<float *>(smem + L.dp);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L.bar);
    __shared__ int abort_flag;

    const float2 *tsrc = xb ? it.tabx : it.taby;
    const size_t img_stride = (size_t)nline * rs;          // float2 per image
    const uint32_t tab_bytes = (uint32_t)(rs * sizeof(float2));
    const uint32_t rec_bytes = (uint32_t)sizeof(DdLine);
    const uint32_t tx_bytes = nb * tab_bytes + rec_bytes + (GEOM == DD_GEOM_PARA ? rec_bytes : 0);

    if (tid == 0) abort_flag = 0;
    if (GEOM != DD_GEOM_PARA)
        for (int k = tid; k <= D; k += (NW * 32)) dps[k] = it.dp[(size_t)v * (D + 1) + k];
    __syncthreads();

    auto issue = [&](int line, int buf) {
        dd_mbar_expect_tx(&bar[buf], tx_bytes);
        dd_bulk_g2s(rec + buf, it.lines + (size_t)v * it.nl + line, rec_bytes, &bar[buf]);
        if (GEOM == DD_GEOM_PARA)
            dd_bulk_g2s(drec + buf, it.dlines + (size_t)v * it.nl + line, rec_bytes, &bar[buf]);
        for (int b = 0; b < nb; b++)
            dd_bulk_g2s(tab + ((size_t)buf * BI + b) * rsmax,
                        tsrc + (size_t)(b0 + b) * img_stride + (size_t)line * rs, tab_bytes, &bar[buf]);
    };

    const int npass = (D + NW * kBinsPerWarp - 1) / (NW * kBinsPerWarp);
    constexpr int kMaxPass = NPASS;   // D <= NPASS * 248 detector bins
    float acc[kMaxPass][BI];
#pragma unroll
    for (int m = 0; m < kMaxPass; m++)
#pragma unroll
        for (int b = 0; b < BI; b++) acc[m][b] = 0.0f;

    const float para_beta = xb ? FDIV(g.pix_y, g.det_size) : FDIV(g.pix_x, g.det_size);
    // fan beams: each pass's detector boundary is the same for all the lines
    // of the view; read it once
    float ud[kMaxPass];
#pragma unroll
    for (int m = 0; m < kMaxPass; m++)
        ud[m] = (GEOM != DD_GEOM_PARA && m < npass) ? dps[min(m * (NW * kBinsPerWarp) + warp * kBinsPerWarp + lane, D)]
                                                     : 0.0f;
    // the last warp issues the copies: the first warps build the piece
    // constants right after the barrier, on every line's critical path
    const int issuer = (NW - 1) * 32;
    if (tid == issuer && rank < nline) issue(rank, 0);
    for (int line = rank, step = 0; line < nline; line += CL, step++) {
        const int buf = step & 1;
        if (!dd_mbar_wait(&bar[buf], ph.parity(buf))) abort_flag = 1;
        ph.flip(buf);
        // past this barrier every warp has finished line - 1, whose buffer
        // takes the copies of line + 1
        __syncthreads();
        if (abort_flag) {
            // this line's copies may still be in flight (the next line's are
            // issued only after this wait): let them land before returning
            if (tid == issuer) dd_mbar_drain(&bar[buf], ph.parity(buf) ^ 1u);
            break;
        }
        if (tid == issuer && line + CL < nline) issue(line + CL, buf ^ 1);
        const DdLine &R = rec[buf];
        const int np = R.h.npiece;
        if (WEIGHTED && np > 0) {
            // BackProjTransWeighted: multiply every pixel by its FBP weight at
            // this view (FanFlatDisCPU2d.cpp:693, FanArcDisCPU2d.cpp:703) and
            // rebuild the line's prefix table in place: warp b scans image b
            // in 128-pixel chunks (4 consecutive pixels per lane, weights in
            // registers), then builds that image's piece constants below, so
            // the rebuild needs no CTA barrier.
            if (warp < nb) {
                float2 *t = tab + ((size_t)buf * BI + warp) * rsmax;
                const float lpos = xb
                    ? pix_centre(0.5f * (float)g.height - (float)line - 0.5f, g.pix_y, g.pix_yshift)
                    : pix_centre((float)line - 0.5f * (float)g.width + 0.5f, g.pix_x, g.pix_xshift);
                const float pitch = xb ? g.pix_x : g.pix_y;
                float carry = 0.0f;
                // 128-pixel chunks, 4 consecutive pixels per lane (two 16-byte
                // loads; rows are 16-byte aligned and rsmax is even)
                for (int k0 = 0; k0 < npix; k0 += 128) {
                    const int i0 = k0 + 4 * lane;
                    float y[4];
                    if (i0 + 3 < npix) {
                        const float4 p01 = *reinterpret_cast<const float4 *>(t + i0);
                        const float4 p23 = *reinterpret_cast<const float4 *>(t + i0 + 2);
                        y[0] = p01.y; y[1] = p01.w; y[2] = p23.y; y[3] = p23.w;
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; e++) y[e] = (i0 + e < npix) ? t[i0 + e].y : 0.0f;
                    }
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float pc = pix_centre((float)(i0 + e) + 0.5f, pitch, vw.axis0);
                        y[e] *= xb ? fan_fbp_weight<GEOM>(vw.srcx, vw.srcy, pc, lpos, g.iso_source)
                                   : fan_fbp_weight<GEOM>(vw.srcx, vw.srcy, lpos, pc, g.iso_source);
                    }
                    const float r1 = y[0] + y[1], r2 = r1 + y[2], r3 = r2 + y[3];
                    float inc = r3;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const float z = __shfl_up_sync(0xffffffffu, inc, o);
                        if (lane >= o) inc += z;
                    }
                    float prev = __shfl_up_sync(0xffffffffu, inc, 1);
                    if (lane == 0) prev = 0.0f;
                    const float base = carry + prev;
                    const float pre[4] = {base, base + y[0], base + r1, base + r2};
                    if (i0 + 3 < npix) {
                        *reinterpret_cast<float4 *>(t + i0) = make_float4(pre[0], y[0], pre[1], y[1]);
                        *reinterpret_cast<float4 *>(t + i0 + 2) = make_float4(pre[2], y[2], pre[3], y[3]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; e++)
                            if (i0 + e < npix) t[i0 + e] = make_float2(pre[e], y[e]);
                    }
                    carry += __shfl_sync(0xffffffffu, inc, 31);
                }
                if (lane == 0) t[npix] = make_float2(carry, 0.0f);
                __syncwarp();   // the piece constants read other lanes' entries
            }
        }
        if (np > 0) {
            const float2 *tb = tab + (size_t)buf * BI * rsmax;
            // warp b: image b's piece constants (for BackProjTransWeighted the
            // warp that rebuilt its table)
            for (int b = warp; b < nb; b += NW) kt[b * 32 + lane] = piece_K(R, tb + (size_t)b * rsmax, lane);
            __syncthreads();
            const float scale = (op == DD_OP_PROJ) ? 1.0f : R.h.alpha;
            const float bound0 = R.h.bound0, endv = R.h.endv;
            const int idet0 = R.h.idet0;
#pragma unroll
            for (int m = 0; m < kMaxPass; m++) {
                if (m >= npass) break;
                const int kb = m * (NW * kBinsPerWarp) + warp * kBinsPerWarp + lane;
                float u;
                if (kb <= idet0) {
                    u = bound0;   // lower boundary of bin idet0 is the walk start
                } else if (GEOM == DD_GEOM_PARA) {
                    const DdLine &Rd = drec[buf];
                    const int idx = min(kb - 1, D - 1);
                    const float est = Rd.p[0].Q + (float)(idx - Rd.p[0].gb) * Rd.p[0].dl;
                    u = (Rd.h.npiece > 0) ? dd_boundary(&Rd, idx, est) : bound0;
                } else {
                    u = ud[m];
                }
                u = fminf(fmaxf(u, bound0), endv);
                // 32 boundaries clamped to the same end of the walk give 31
                // zero differences: the warp skips the bins this line misses
                if (__all_sync(0xffffffffu, u == bound0) || __all_sync(0xffffffffu, u == endv)) continue;
                const Loc lc = locate(R, u);
#pragma unroll
                for (int b = 0; b < BI; b++) {
                    if (b < nb) {
                        const float2 e = tb[(size_t)b * rsmax + lc.j];
                        const float f = fmaf(lc.r, e.y, fmaf(lc.dl, e.x, kt[b * 32 + lc.p]));
                        const float fn = __shfl_down_sync(0xffffffffu, f, 1);
                        if (lane < kBinsPerWarp) acc[m][b] = fmaf(scale, fn - f, acc[m][b]);
                    }
                }
            }
        }
    }
    // no copy is left in flight here: the next line's copies are issued only
    // after its predecessor's wait succeeded, and an abort drained its line's
    __syncthreads();   // the next item's first copies reuse the buffers
    if constexpr (CL > 1) {
        // ranks > 0 leave their sums in the (idle) line-table space; rank 0
        // adds them in rank order, so the result does not depend on timing
        cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
        float *red = reinterpret_cast<float *>(smem + L.tab);
        if (rank != 0 && !abort_flag) {
#pragma unroll
            for (int m = 0; m < kMaxPass; m++) {
                if (m >= npass) break;
#pragma unroll
                for (int b = 0; b < BI; b++) red[(m * BI + b) * (NW * 32) + tid] = acc[m][b];
            }
        }
        cluster.sync();
        int ab = 0;
        for (int r = 0; r < CL; r++) ab |= *cluster.map_shared_rank(&abort_flag, r);
        if (rank == 0 && !ab) {
            for (int r = 1; r < CL; r++) {
                const float *rr = cluster.map_shared_rank(red, r);
#pragma unroll
                for (int m = 0; m < kMaxPass; m++) {
                    if (m >= npass) break;
#pragma unroll
                    for (int b = 0; b < BI; b++) acc[m][b] += rr[(m * BI + b) * (NW * 32) + tid];
                }
            }
        }
        cluster.sync();   // no rank leaves (or reuses its buffers) before rank 0 has read them
        if (ab) return false;
        if (rank != 0) return true;
    } else {
        if (abort_flag) return false;
    }
#pragma unroll
    for (int m = 0; m < kMaxPass; m++) {
        if (m >= npass) break;
        const int k = m * (NW * kBinsPerWarp) + warp * kBinsPerWarp + lane;
        if (lane < kBinsPerWarp && k < D) {
            float beta = 1.0f;
            if (op == DD_OP_PROJ) beta = (GEOM == DD_GEOM_PARA) ? para_beta : it.bcoef[(size_t)v * (D + 1) + k];
            const int ko = vw.flip ? D - 1 - k : k;
#pragma unroll
            for (int b = 0; b < BI; b++) {   // static indices keep acc in registers
                if (b >= nb) break;
                const size_t o = ((size_t)(b0 + b) * it.V + v) * D + ko;
                // rounded product, then rounded difference: bit-equal to a
                // separate projection followed by a subtraction (no FMA)
                float val = __fmul_rn(acc[m][b], beta);
                if (it.sub) val = __fsub_rn(val, it.sub[o]);
                it.out[o] = val;
            }
        }
    }
    return true;
}

__device__ __forceinline__ void init_bars(uint64_t *bar, int n = 2) {
    if (threadIdx.x == 0) {
        for (int i = 0; i < n; i++) dd_mbar_init(&bar[i], 1);
        dd_fence_mbar_init();
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Adjoint-type kernel (ProjTrans, BackProj, BackProjWeighted): pixel gathers.
// CTA = 32x32 image tile x kBI images; loops over all views, accumulating in
// registers (row-major ownership for x-branch views, column-major for
// y-branch views, merged through shared memory at the end).
// ---------------------------------------------------------------------------
constexpr int kLinesPerWarp = kTile / kWarps;   // 4

// Fan: integral of the detector function up to u (clamped) for image b.
__device__ __forceinline__ void det_index_fan(int geom, const dd_geom2d &g, const DdView2 &vw,
                                              float view, float u, int *kk) {
    const int D = g.num_det;
    float kf;
    if (geom == DD_GEOM_FLAT) {
        const float R = g.iso_source;
        const float vds = FMUL(FDIV(R, g.source_detector), g.det_size);
        const float vbs = FMUL(FDIV(R, g.source_detector), g.bin_shift);
        // virtual-detector coordinate of the ray source -> (u on the axis)
        const float t = vw.xb ? R * u * vw.c / (R + u * vw.s) : R * u * vw.s / (R - u * vw.c);
        const float q = (t - vbs) / vds;
        kf = vw.flip ? (float)D * 0.5f - q : q + (float)D * 0.5f;
    } else {
        // arc: angle of the ray through the axis point
        float ang = vw.xb ? atan2f(u - vw.srcx, vw.srcy) : 1.5707963267948966f - atanf((u - vw.srcy) / vw.srcx);
        const float base = view + g.bin_shift;
        ang += 3.14159265358979f * rintf((base - ang) * 0.3183098861837907f);
        const float q = (ang - base) / g.det_size;
        kf = vw.flip ? (float)D * 0.5f - q : q + (float)D * 0.5f;
    }
    int k = (int)floorf(kf);
    *kk = min(max(k, 0), D - 1);
}

// Detector-table entries per image staged in shared memory for one view
// (fan beams): the bins a 32x32 tile can touch.  Views whose range is wider
// gather from global memory instead.
constexpr int kStage = 256;

// Views in flight in the fan-beam adjoint: the copies of view v + 2 are issued
// while view v is computed (part of the map comes from HBM).
constexpr int kAdjBufs = 3;

static_assert((kAdjBufs * kMapBlkBytes + kAdjBufs * kBI * kStage * 8) % 16 == 0,
              "the fan adjoint's per-buffer copy descriptors must be 16-byte aligned");

// Shared-memory layout of the adjoint kernel (bytes).  Parallel beam: line
// records (and detector-side records); fan beams: adjoint-map rows, detector
// table slices and per-line scales.
struct AdjSmem {
    int rec, drec, kd, stage, krange, bar, total;
    int map;
};

__host__ __device__ inline AdjSmem adj_smem(int geom) {
    AdjSmem s;
    int o = 0;
    s.map = 0;
    if (geom != DD_GEOM_PARA) {
        s.rec = s.drec = s.kd = 0;
        s.map = o; o += kAdjBufs * kMapBlkBytes;
        s.stage = o; o += kAdjBufs * kBI * kStage * (int)sizeof(float2);
        s.krange = o; o += 4 * kAdjBufs * (int)sizeof(int);   // 16-byte aligned: read as int4
        s.bar = o; o += kAdjBufs * (int)sizeof(uint64_t);
        s.total = (o + 127) & ~127;
        return s;
    }
    s.rec = o; o += 2 * kTile * (int)sizeof(DdLine);
    s.drec = o; if (geom == DD_GEOM_PARA) o += 2 * kTile * (int)sizeof(DdLine);
    s.kd = o; if (geom == DD_GEOM_PARA) o += kWarps * kBI * 32 * (int)sizeof(float);
    s.stage = o; if (geom != DD_GEOM_PARA) o += 2 * kBI * kStage * (int)sizeof(float2);
    s.krange = o; o += 4 * (int)sizeof(int);
    s.bar = o; o += 2 * (int)sizeof(uint64_t);
    // the final merge of the two pixel ownerships reuses the record buffers
    const int merge = kBI * kTile * (kTile + 1) * (int)sizeof(float);
    if (o < merge + 16) o = merge + 16;
    s.total = (o + 127) & ~127;
    return s;
}

// Detector bins [kmin, kmax] that pixels of the tile at (c0, r0) can reach at
// one view (fan beams): the walked pixel boundaries lie inside the tile's
// rectangle, whose central projection onto the axis spans the projections of
// its four corners.  Two bins of margin absorb rounding.
__device__ __forceinline__ void tile_bin_range(int geom, const dd_geom2d &g, const DdView2 &vw, float view, int c0,
                                               int r0, int *kmin, int *kmax) {
    const int W = g.width, H = g.height;
    const float xs[2] = {((float)c0 - 0.5f * W) * g.pix_x + g.pix_xshift,
                         ((float)min(c0 + kTile, W) - 0.5f * W) * g.pix_x + g.pix_xshift};
    const float ys[2] = {(0.5f * H - (float)r0) * g.pix_y + g.pix_yshift,
                         (0.5f * H - (float)min(r0 + kTile, H)) * g.pix_y + g.pix_yshift};
    int lo = g.num_det, hi = -1;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float px = xs[i & 1], py = ys[i >> 1];
        const float u = vw.xb ? dd_map2x(vw.srcx, vw.srcy, px, py) : dd_map2y(vw.srcx, vw.srcy, px, py);
        int k;
        det_index_fan(geom, g, vw, view, u, &k);
        lo = min(lo, k);
        hi = max(hi, k);
    }
    *kmin = max(lo - 2, 0);
    *kmax = min(hi + 2, g.num_det - 1);
}

// Detector-table position of axis value uu (fan beams): bin k with
// d_k <= uu < d_{k+1} (corrected against the exact table), clamped to the
// walked bins.  Returns k and d_k.
__device__ __forceinline__ int fan_bin(int geom, const dd_geom2d &g, const DdView2 &vw, float view,
                                       const float *__restrict__ dpv, float uu, int idet0, float *dk_out) {
    const int D = g.num_det;
    int k;
    det_index_fan(geom, g, vw, view, uu, &k);
    float dk = __ldg(dpv + k);
    if (k > 0 && uu < dk) {
        k--;
        dk = __ldg(dpv + k);
    } else if (k < D - 1 && uu >= __ldg(dpv + k + 1)) {
        k++;
        dk = __ldg(dpv + k);
    }
    if (k < idet0) {
        k = idet0;
        dk = __ldg(dpv + k);
    }
    *dk_out = dk;
    return k;
}

// One adjoint work item: a 32x32 tile of one instance and a group of <= kBI
// of its images, accumulated over all views.  Epilogue: out = value, or
// out = base + scale * value (base may alias out: in-place update).
struct AdjItem {
    int c0, r0, b0, nb, V, nl;
    const float *angles;
    const DdView2 *views;
    const float *dp;
    const DdLine *lines, *dlines;
    const unsigned char *amap;   // fan beams: adjoint-map blocks (plan)
    const int2 *trange;          // fan beams, per (view, tile): {first staged bin, bins | xb << 16} (plan)
    const float2 *dtab;          // detector tables of image 0 of the instance
    float *out;                  // image 0 of the instance
    const float *base;
    float scale;
};

template <int GEOM, int OPK>   // OPK: 0 ProjTrans, 1 BackProj, 2 BackProjWeighted
__device__ bool adj_tile(const dd_geom2d &g, const AdjItem &it, unsigned char *smem, DdPhases &ph) {
    const AdjSmem SL = adj_smem(GEOM);
    const int V = it.V, nl = it.nl;
    const float *__restrict__ angles = it.angles;
    const DdView2 *__restrict__ views = it.views;
    const float *__restrict__ dp = it.dp;
    const DdLine *__restrict__ lines = it.lines;
    const DdLine *__restrict__ dlines = it.dlines;
    const float2 *__restrict__ dtab = it.dtab;
    DdLine *recs = reinterpret_cast<DdLine *>(smem + SL.rec);
    DdLine *drecs = reinterpret_cast<DdLine *>(smem + SL.drec);
    float *kdp = reinterpret_cast<float *>(smem + SL.kd);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + SL.bar);
    float2 *stage = reinterpret_cast<float2 *>(smem + SL.stage);
    int *krange = reinterpret_cast<int *>(smem + SL.krange);   // per buffer: first staged bin, count
    __shared__ int abort_flag;

    const int c0 = it.c0, r0 = it.r0;
    const int b0 = it.b0;
    const int nb = it.nb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = g.width, H = g.height, D = g.num_det;
    const int rsd = rs_entries(D);

    if (tid == 0) abort_flag = 0;
    __syncthreads();

    // records of the tile's lines of view v: rows r0.. (x-branch) or columns c0..
    // plus, for fan beams, the slice of every image's detector table that the
    // tile can reach (16-byte aligned: even first bin, even count)
    auto issue = [&](int v, int buf) {
        const DdView2 vwv = views[v];
        const int xbv = vwv.xb;
        const int line0 = xbv ? r0 : c0;
        const int nline = xbv ? H : W;
        const int n = min(kTile, nline - line0);
        const uint32_t bytes = (uint32_t)(n * sizeof(DdLine));
        uint32_t tx = bytes * (GEOM == DD_GEOM_PARA ? 2u : 1u);
        int kb = 0, kn = 0;
        if (GEOM != DD_GEOM_PARA) {
            int kmin, kmax;
            tile_bin_range(GEOM, g, vwv, angles[v], c0, r0, &kmin, &kmax);
            kb = kmin & ~1;
            kn = (kmax - kb + 2) & ~1;
            if (kb + kn > rsd) kn = rsd - kb;
            if (kn > kStage || kn <= 0) kn = 0;
            tx += (uint32_t)(nb * kn * (int)sizeof(float2));
        }
        krange[2 * buf] = kb;
        krange[2 * buf + 1] = kn;
        dd_mbar_expect_tx(&bar[buf], tx);
        dd_bulk_g2s(recs + buf * kTile, lines + (size_t)v * nl + line0, bytes, &bar[buf]);
        if (GEOM == DD_GEOM_PARA)
            dd_bulk_g2s(drecs + buf * kTile, dlines + (size_t)v * nl + line0, bytes, &bar[buf]);
        if (kn > 0)
            for (int b = 0; b < nb; b++)
                dd_bulk_g2s(stage + ((size_t)buf * kBI + b) * kStage, dtab + ((size_t)(b0 + b) * V + v) * rsd + kb,
                            (uint32_t)(kn * sizeof(float2)), &bar[buf]);
    };

    float ax[kLinesPerWarp][kBI], ay[kLinesPerWarp][kBI];
#pragma unroll
    for (int q = 0; q < kLinesPerWarp; q++)
#pragma unroll
        for (int b = 0; b < kBI; b++) ax[q][b] = ay[q][b] = 0.0f;

    if (tid == 0) issue(0, 0);
    int inflight = -1;
    for (int v = 0; v < V; v++) {
        const int buf = v & 1;
        if (tid == 0 && v + 1 < V) issue(v + 1, buf ^ 1);
        if (!dd_mbar_wait(&bar[buf], ph.parity(buf))) abort_flag = 1;
        ph.flip(buf);
        __syncthreads();
        if (abort_flag) {
            // view v's copies (not waited for) and view v + 1's may be in flight
            if (tid == 0) dd_mbar_drain(&bar[buf], ph.parity(buf) ^ 1u);
            inflight = (v + 1 < V) ? (buf ^ 1) : -1;
            break;
        }
        const DdView2 vw = views[v];
        const float view = angles[v];
        const float *dpv = dp + (size_t)v * (D + 1);
        const float dend = (GEOM == DD_GEOM_PARA) ? 0.0f : __ldg(dpv + D);
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) {
            const int rel = warp + kWarps * q;
            int line, pi;
            if (vw.xb) {
                line = r0 + rel;
                pi = c0 + lane;
                if (line >= H) continue;
            } else {
                line = c0 + rel;
                pi = H - r0 - kTile + lane;
                if (line >= W) continue;
            }
            const DdLine &L = recs[buf * kTile + rel];
            const int np = L.h.npiece;
            if (np == 0) continue;   // warp-uniform
            const int i0 = L.h.i0, nend = L.h.nend;
            const float bound0 = L.h.bound0;
            const int idet0 = L.h.idet0;
            const bool valid = (pi >= i0) && (pi < nend) && (pi >= 0);
            const bool need_low = valid && (lane == 0 || pi == i0);
            // image-independent geometry: boundary values and their detector positions
            float up = bound0, low = bound0;
            if (valid) up = dd_boundary(&L, pi, L.p[0].Q + (float)(pi - L.p[0].gb) * L.p[0].dl);
            if (need_low && pi > i0) low = dd_boundary(&L, pi - 1, L.p[0].Q + (float)(pi - 1 - L.p[0].gb) * L.p[0].dl);
            const float alpha = (OPK == 0) ? 1.0f : L.h.alpha;
            float wgt = alpha;
            if (OPK == 2 && valid) {
                float pcx, pcy;
                if (vw.xb) {
                    pcx = pix_centre((float)pi + 0.5f, g.pix_x, vw.axis0);
                    pcy = pix_centre(0.5f * (float)H - (float)line - 0.5f, g.pix_y, g.pix_yshift);
                } else {
                    pcx = pix_centre((float)line - 0.5f * (float)W + 0.5f, g.pix_x, g.pix_xshift);
                    pcy = pix_centre((float)pi + 0.5f, g.pix_y, vw.axis0);
                }
                wgt = alpha * fan_fbp_weight<GEOM>(vw.srcx, vw.srcy, pcx, pcy, g.iso_source);
            }
            if (GEOM == DD_GEOM_PARA) {
                const DdLine &Ld = drecs[buf * kTile + rel];
                const int npd = Ld.h.npiece;
                float *kd = kdp + warp * kBI * 32;
                for (int b = 0; b < nb; b++) {
                    const float Kb = npd > 0 ? piece_K(Ld, dtab + ((size_t)(b0 + b) * V + v) * rsd, lane) : 0.0f;
                    kd[b * 32 + lane] = Kb;
                }
                __syncwarp();
                int pU = 0, jU = 0, pL = 0, jL = 0;
                float rU = 0.0f, rL = 0.0f, dlU = 0.0f, dlL = 0.0f;
                if (npd > 0) {
                    const float uu = fminf(fmaxf(up, bound0), Ld.h.endv);
                    dd_locate(&Ld, uu, &pU, &jU, &rU);
                    dlU = Ld.p[pU].dl;
                    const float ul = fminf(fmaxf(low, bound0), Ld.h.endv);
                    dd_locate(&Ld, ul, &pL, &jL, &rL);
                    dlL = Ld.p[pL].dl;
                }
#pragma unroll
                for (int b = 0; b < kBI; b++) {
                    if (b >= nb) break;
                    const float2 *t = dtab + ((size_t)(b0 + b) * V + v) * rsd;   // per image
                    float hu = 0.0f, hl2 = 0.0f;
                    if (npd > 0) {
                        const float2 e = __ldg(t + jU);
                        hu = fmaf(rU, e.y, fmaf(dlU, e.x, kd[b * 32 + pU]));
                        if (need_low) {
                            const float2 e2 = __ldg(t + jL);
                            hl2 = fmaf(rL, e2.y, fmaf(dlL, e2.x, kd[b * 32 + pL]));
                        }
                    }
                    float hl = __shfl_up_sync(0xffffffffu, hu, 1);
                    if (need_low) hl = hl2;
                    if (valid) {
                        const float val = wgt * (hu - hl);
                        if (vw.xb) ax[q][b] += val;
                        else ay[q][b] += val;
                    }
                }
                __syncwarp();
            } else {
                const float uu = fminf(fmaxf(up, bound0), dend);
                float dkU;
                const int kU = fan_bin(GEOM, g, vw, view, dpv, uu, idet0, &dkU);
                const float offU = uu - dkU;
                int kL = kU;
                float offL = 0.0f;
                if (need_low) {
                    const float ul = fminf(fmaxf(low, bound0), dend);
                    float dkL;
                    kL = fan_bin(GEOM, g, vw, view, dpv, ul, idet0, &dkL);
                    offL = ul - dkL;
                }
                const int kb = krange[2 * buf], kn = krange[2 * buf + 1];
                const bool inU = (unsigned)(kU - kb) < (unsigned)kn;
                const bool inL = (unsigned)(kL - kb) < (unsigned)kn;
                const float2 *sb = stage + (size_t)buf * kBI * kStage;
#pragma unroll
                for (int b = 0; b < kBI; b++) {
                    if (b >= nb) break;
                    const float2 *t = dtab + ((size_t)(b0 + b) * V + v) * rsd;   // per image
                    const float2 e = inU ? sb[b * kStage + (kU - kb)] : __ldg(t + kU);
                    const float hu = fmaf(offU, e.y, e.x);
                    float hl = __shfl_up_sync(0xffffffffu, hu, 1);
                    if (need_low) {
                        const float2 e2 = inL ? sb[b * kStage + (kL - kb)] : __ldg(t + kL);
                        hl = fmaf(offL, e2.y, e2.x);
                    }
                    if (valid) {
                        const float val = wgt * (hu - hl);
                        if (vw.xb) ax[q][b] += val;
                        else ay[q][b] += val;
                    }
                }
            }
        }
        __syncthreads();   // buffer `buf` is refilled by the next iteration's issue
    }
    if (abort_flag) {
        if (tid == 0 && inflight >= 0) dd_mbar_drain(&bar[inflight], ph.parity(inflight));
        if (inflight >= 0) ph.flip(inflight);
        __syncthreads();
        return false;
    }
    // merge the two ownerships through shared memory (reusing the record buffers)
    float (*tile)[kTile][kTile + 1] = reinterpret_cast<float (*)[kTile][kTile + 1]>(smem + SL.rec);
    // (b loops unrolled over kBI: static indices keep ax / ay in registers)
#pragma unroll
    for (int b = 0; b < kBI; b++) {
        if (b >= nb) break;
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) tile[b][warp + kWarps * q][lane] = ax[q][b];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < kBI; b++) {
        if (b >= nb) break;
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) tile[b][kTile - 1 - lane][warp + kWarps * q] += ay[q][b];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < kBI; b++) {
        if (b >= nb) break;
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) {
            const int r = r0 + warp + kWarps * q, c = c0 + lane;
            if (r < H && c < W) {
                const size_t o = ((size_t)(b0 + b) * H + r) * W + c;
                const float val = tile[b][warp + kWarps * q][lane];
                it.out[o] = it.base ? fmaf(it.scale, val, it.base[o]) : val;
            }
        }
    }
    __syncthreads();   // the tile buffer aliases the record buffers of the next item
    return true;
}


// ---------------------------------------------------------------------------
// Fan-beam adjoint through the adjoint map.  For every view the CTA copies by
// TMA, for its 32 walked lines, the map entries {bin, offset} of the tile's
// pixel boundaries, the per-line scales and the slice of every image's
// detector prefix table the tile can reach.  A thread owns fixed pixels (4
// consecutive rows of one column: warp = row group, lane = column) for every
// view, so one set of accumulators serves both projection axes: pixel value
// += w (H(upper) - H(lower)), with H(u) = G_k + (u - d_k) g_k read at the two
// staged boundary entries (for views that walk columns the 4 pixels share
// boundaries: 5 values of H serve them).
// ---------------------------------------------------------------------------
template <int GEOM, int OPK>   // OPK: 0 ProjTrans, 1 BackProj, 2 BackProjWeighted
__device__ bool adj_tile_map(const dd_geom2d &g, const AdjItem &it, unsigned char *smem, DdPhases &ph) {
    const AdjSmem SL = adj_smem(GEOM);
    const int V = it.V;
    const int W = g.width, H = g.height, D = g.num_det;
    const int rsd = rs_entries(D);
    unsigned char *mapb = smem + SL.map;                           // [kAdjBufs] map blocks
    float2 *stage = reinterpret_cast<float2 *>(smem + SL.stage);   // [kAdjBufs][kBI][kStage]
    int *krange = reinterpret_cast<int *>(smem + SL.krange);       // per buffer: first bin, bins, first entry
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + SL.bar);
    __shared__ int abort_flag;
    const int c0 = it.c0, r0 = it.r0, b0 = it.b0, nb = it.nb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float2 *__restrict__ dtab = it.dtab;
    if (tid == 0) abort_flag = 0;
    __syncthreads();

    // What view v's copies move, from its staged range {first bin, bins | xb << 16}.
    struct Cp {
        int xb, elo, kb, kn;
    };
    const int tile = (r0 / kTile) * tiles_x(&g) + c0 / kTile, ntiles = tiles_n(&g);
    auto desc = [&](int2 tr) {
        Cp d;
        d.xb = tr.y >> 16;
        d.elo = map_first(&g, d.xb, c0, r0);
        d.kb = tr.x;
        d.kn = tr.y & 0xFFFF;
        return d;
    };
    // thread 0 arms a buffer's barrier with the byte count of its next view,
    // before any warp issues a copy into it
    auto arm = [&](int buf, const Cp &d) {
        dd_mbar_expect_tx(&bar[buf], (uint32_t)(kMapBlkBytes + nb * d.kn * (int)sizeof(float2)));
    };
    // View v's copies, one per warp: warp 0 moves the tile's map block, warp
    // b + 1 (b < nb) the detector-table slice of image b.
    auto issue = [&](int v, int buf, const Cp &d) {
        if (tid == 0) {
            krange[4 * buf] = d.kb;
            krange[4 * buf + 1] = d.kn;
            krange[4 * buf + 2] = d.elo;
            krange[4 * buf + 3] = d.xb;
        }
        if (lane == 0) {
            if (warp == 0)
                dd_bulk_g2s(mapb + (size_t)buf * kMapBlkBytes, it.amap + ((size_t)v * ntiles + tile) * kMapBlkBytes,
                            (uint32_t)kMapBlkBytes, &bar[buf]);
            else if (warp <= nb && d.kn > 0)
                dd_bulk_g2s(stage + ((size_t)buf * kBI + warp - 1) * kStage,
                            dtab + ((size_t)(b0 + warp - 1) * V + v) * rsd + d.kb, (uint32_t)(d.kn * sizeof(float2)),
                            &bar[buf]);
        }
    };

    float acc[kLinesPerWarp][kBI];
#pragma unroll
    for (int q = 0; q < kLinesPerWarp; q++)
#pragma unroll
        for (int b = 0; b < kBI; b++) acc[q][b] = 0.0f;

    {
        const Cp d0 = desc(it.trange[tile]);
        const Cp d1 = desc(V > 1 ? it.trange[(size_t)ntiles + tile] : make_int2(0, 0));
        if (tid == 0) {
            arm(0, d0);
            if (V > 1) arm(1, d1);
        }
        __syncthreads();
        issue(0, 0, d0);
        if (V > 1) issue(1, 1, d1);
    }
    // only the warps that issue a view's copies (warp 0: the map block, warps
    // 1 .. nb: the detector slices) need its descriptor
    const bool issuing = warp <= nb;
    int2 tr_next = (V > 2 && issuing) ? it.trange[(size_t)2 * ntiles + tile] : make_int2(0, 0);   // view v + 2
    int vstop = V;   // first view not waited for (the copies of vstop may be in flight)
    int buf = 0, buf2 = 2 % kAdjBufs;   // buffers of views v and v + 2
    for (int v = 0; v < V; v++, buf = (buf + 1 == kAdjBufs) ? 0 : buf + 1,
                                buf2 = (buf2 + 1 == kAdjBufs) ? 0 : buf2 + 1) {
        const bool more = v + 2 < V;
        Cp dn;
        if (more && issuing) {
            dn = desc(tr_next);
            // the phase of view v - 1 on this barrier was waited for before the
            // previous barrier, so it can be armed for view v + 2 now
            if (tid == 0) arm(buf2, dn);
        }
        if (!dd_mbar_wait(&bar[buf], ph.parity(buf))) abort_flag = 1;
        ph.flip(buf);
        // one barrier per view: past it every warp has finished view v - 1
        __syncthreads();
        if (abort_flag) {
            // view v's copies (not waited for) may still be in flight
            if (tid == 0) dd_mbar_drain(&bar[buf], ph.parity(buf) ^ 1u);
            vstop = v + 1;
            break;
        }
        // so the copies of view v + 2 go into the buffer of view v - 1
        if (more && issuing) {
            issue(v + 2, buf2, dn);
            if (v + 3 < V) tr_next = it.trange[(size_t)(v + 3) * ntiles + tile];
        }
        const int4 kr = reinterpret_cast<const int4 *>(krange)[buf];   // one 16-byte load
        const int kb = kr.x, kn = kr.y, elo = kr.z, xb = kr.w;
        const int2 *mp = reinterpret_cast<const int2 *>(mapb + (size_t)buf * kMapBlkBytes);
        const float *alb = reinterpret_cast<const float *>(mp + kTile * kMapE);   // line scales
        const float2 *sb = stage + (size_t)buf * kBI * kStage;
        DdView2 vw;   // BackProjWeighted: the view's source and first pixel edge
        if (OPK == 2) vw = it.views[v];
        // this thread's pixels: rows rq0 .. rq0 + 3 of column c
        const int rq0 = r0 + kLinesPerWarp * warp, c = c0 + lane;
        if (!xb) {
            // views that walk columns: the thread's 4 pixels are consecutive
            // on its line and pixel q's lower boundary is pixel q + 1's upper
            // one, so 5 boundary values serve the 4 pixels (the same values:
            // results are unchanged)
            const int nv = (c < W) ? min(kLinesPerWarp, H - rq0) : 0;
            if (nv > 0) {
                const int lr = c - c0, E = H - rq0 - elo;   // pixel q: upper entry E - q, lower E - q - 1
                int2 m[kLinesPerWarp + 1];
                bool all_in = true;   // every used entry in the staged slice (the usual case)
#pragma unroll
                for (int i = 0; i <= kLinesPerWarp; i++) {
                    m[i] = (i <= nv) ? mp[lr * kMapE + E - i] : make_int2(-1, 0);
                    if (m[i].x >= 0 && (unsigned)(m[i].x - kb) >= (unsigned)kn) all_in = false;
                }
                float wq[kLinesPerWarp];
#pragma unroll
                for (int q = 0; q < kLinesPerWarp; q++) {
                    float wgt = (OPK == 0) ? 1.0f : alb[lr];
                    if (OPK == 2) {
                        const float pcx = pix_centre((float)c - 0.5f * (float)W + 0.5f, g.pix_x, g.pix_xshift);
                        const float pcy = pix_centre((float)(H - 1 - (rq0 + q)) + 0.5f, g.pix_y, vw.axis0);
                        wgt = wgt * fan_fbp_weight<GEOM>(vw.srcx, vw.srcy, pcx, pcy, g.iso_source);
                    }
                    wq[q] = wgt;
                }
#pragma unroll
                for (int b = 0; b < kBI; b++) {
                    if (b >= nb) break;
                    const float2 *t = dtab + ((size_t)(b0 + b) * V + v) * rsd;   // per image
                    float h[kLinesPerWarp + 1];
                    if (all_in) {
#pragma unroll
                        for (int i = 0; i <= kLinesPerWarp; i++) {
                            const float2 e = sb[b * kStage + max(m[i].x - kb, 0)];
                            h[i] = fmaf(__int_as_float(m[i].y), e.y, e.x);   // unused where m[i].x < 0
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i <= kLinesPerWarp; i++) {
                            h[i] = 0.0f;
                            if (m[i].x >= 0) {
                                const bool in = (unsigned)(m[i].x - kb) < (unsigned)kn;
                                const float2 e = in ? sb[b * kStage + (m[i].x - kb)] : __ldg(t + m[i].x);
                                h[i] = fmaf(__int_as_float(m[i].y), e.y, e.x);
                            }
                        }
                    }
#pragma unroll
                    for (int q = 0; q < kLinesPerWarp; q++)
                        if (q < nv && m[q].x >= 0 && m[q + 1].x >= 0) acc[q][b] += wq[q] * (h[q] - h[q + 1]);
                }
            }
        } else {
#pragma unroll
            for (int q = 0; q < kLinesPerWarp; q++) {
                const int r = rq0 + q;
                if (r >= H || c >= W) continue;
                const int lr = r - r0, eu = c + 1 - elo;   // line r, pixel c
                const int2 up = mp[lr * kMapE + eu], low = mp[lr * kMapE + eu - 1];
                if (up.x < 0 || low.x < 0) continue;
                float wgt = (OPK == 0) ? 1.0f : alb[lr];
                if (OPK == 2) {
                    const float pcx = pix_centre((float)c + 0.5f, g.pix_x, vw.axis0);
                    const float pcy = pix_centre(0.5f * (float)H - (float)r - 0.5f, g.pix_y, g.pix_yshift);
                    wgt = wgt * fan_fbp_weight<GEOM>(vw.srcx, vw.srcy, pcx, pcy, g.iso_source);
                }
                const float offU = __int_as_float(up.y), offL = __int_as_float(low.y);
                const bool inU = (unsigned)(up.x - kb) < (unsigned)kn;
                const bool inL = (unsigned)(low.x - kb) < (unsigned)kn;
                if (inU && inL) {   // both entries in the staged slice (the usual case)
                    const float2 *su = sb + (up.x - kb), *sl = sb + (low.x - kb);
#pragma unroll
                    for (int b = 0; b < kBI; b++) {
                        if (b >= nb) break;
                        const float2 e = su[b * kStage], e2 = sl[b * kStage];
                        const float hu = fmaf(offU, e.y, e.x);
                        const float hl = fmaf(offL, e2.y, e2.x);
                        acc[q][b] += wgt * (hu - hl);
                    }
                } else {
#pragma unroll
                    for (int b = 0; b < kBI; b++) {
                        if (b >= nb) break;
                        const float2 *t = dtab + ((size_t)(b0 + b) * V + v) * rsd;   // per image
                        const float2 e = inU ? sb[b * kStage + (up.x - kb)] : __ldg(t + up.x);
                        const float2 e2 = inL ? sb[b * kStage + (low.x - kb)] : __ldg(t + low.x);
                        const float hu = fmaf(offU, e.y, e.x);
                        const float hl = fmaf(offL, e2.y, e2.x);
                        acc[q][b] += wgt * (hu - hl);
                    }
                }
            }
        }
    }
    __syncthreads();   // the next item's first copies reuse the buffers
    if (abort_flag) {
        // let the copies of view vstop (issued, not waited for) land
        for (int u = vstop; u < V && u < vstop + 1; u++) {
            const int b = u % kAdjBufs;
            if (tid == 0) dd_mbar_drain(&bar[b], ph.parity(b));
            ph.flip(b);
        }
        __syncthreads();
        return false;
    }
#pragma unroll
    for (int q = 0; q < kLinesPerWarp; q++) {
        const int r = r0 + kLinesPerWarp * warp + q, c = c0 + lane;
        if (r >= H || c >= W) continue;
#pragma unroll
        for (int b = 0; b < kBI; b++) {   // static indices keep acc in registers
            if (b >= nb) break;
            const size_t o = ((size_t)(b0 + b) * H + r) * W + c;
            it.out[o] = it.base ? fmaf(it.scale, acc[q][b], it.base[o]) : acc[q][b];
        }
    }
    return true;
}


// ---- host launchers shared by both translation units (dd2d.cu) -----------
struct ProfRec;
ProfRec *prof_begin(int kind, cudaStream_t st);
void prof_end(ProfRec *r, cudaStream_t st);
void count_launches(int n);
int plan(int scan, const dd_geom2d *g, const float *angles, int V, void *planp, size_t bytes,
         cudaStream_t st, bool with_map = true);
int validate(int scan, int op, const dd_geom2d *g, int B, int V);
int geom_of(int scan);
int launch_status();
int max_smem_optin();   // largest dynamic shared memory per CTA (opt-in) on this device
// prefix tables of B images (forward) / B sinograms (adjoint) of one geometry
int launch_image_tables(const dd_geom2d *g, const float *in, int B, float2 *tx, float2 *ty, cudaStream_t st);
int launch_det_tables(int geom, int op, const dd_geom2d *g, const char *planb, const float *in, int B,
                      int V, float2 *dtab, cudaStream_t st);

}  // namespace dd2
