// GB300 (sm_103a) 2-D distance-driven projector: parallel, fan-flat, fan-arc.
//
// Replaces the 16 2-D operators of deeprecon's radontorch extension
// (RadonTorch.cpp:17-568; kernels deeprecon/cuda/dis2d/*.cu, CPU path
// deeprecon/cpu/dis2d/*.cpp).  Results follow the reference CPU path, which is
// the parity target.
//
// Algorithm (integral form of the DD merge walk).  For one view and one
// walked image line, deeprecon merges the sorted pixel boundaries b_i and
// detector boundaries d_k on a projection axis and weights every overlap
// segment.  The same sums are differences of integrals:
//   forward (detector gathers):  bin_k  += F(d_{k+1}) - F(d_k),
//                                F(u) = integral of the pixel function to u;
//   adjoint (pixel gathers):     pix_i  += H(b_i) - H(b_{i-1}),
//                                H(u) = integral of the detector function.
// F is evaluated from a per-line prefix table (S_j, x_j) staged in shared
// memory by TMA bulk copies; H from a per-view prefix table of the detector
// row.  Both are branch-free interpolations, so a warp processes 32 adjacent
// boundaries in lock step and neighbouring lanes exchange values with one
// shuffle.  The adjoint is a gather: no atomics, deterministic.
//
// The pixel boundaries are deeprecon's drifted FP32 sequence
// (`Point1Proj += PixInterval`), represented exactly by per-line binade
// pieces (dd_geom.cuh); the integral over a drifted pixel is then
//   F(u) = K_p + dl_p * S_j + r * x_j
// with a per-piece constant K_p computed once per line by a warp scan.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/pridediff_dd.h"
#include "dd_geom2d.cuh"
#include "dd_tma.cuh"

namespace dd2 {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kBinsPerWarp = 31;   // 32 boundaries -> 31 bins per warp pass
constexpr int kBI = 8;             // images per CTA (geometry amortised over them)

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
__host__ __device__ inline int rs_entries(int n) { return (n + 2) & ~1; }   // n+1 float2, 16-B rows

// ---------------------------------------------------------------------------
// Workspace layout
// ---------------------------------------------------------------------------
struct PlanLayout {
    size_t views, ang, dp, bcoef, lines, dlines, total;
    int nl;   // line records per view = max(H, W)
};

static PlanLayout plan_layout(int scan, const dd_geom2d *g, int V) {
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
    L.total = o;
    return L;
}

struct ApplyLayout {
    size_t tabx, taby, dtab, status, total;
};

static bool op_is_forward(int op) {
    return op == DD_OP_PROJ || op == DD_OP_BPROJ_T || op == DD_OP_BPROJ_TW;
}

static ApplyLayout apply_layout(int op, const dd_geom2d *g, int B, int V) {
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
// Plan kernels
// ---------------------------------------------------------------------------
__global__ void k_views(int geom, dd_geom2d g, const float *__restrict__ angles, int V,
                        DdView2 *__restrict__ views, float *__restrict__ ang,
                        float *__restrict__ dp, float *__restrict__ bcoef) {
    const int v = blockIdx.x;
    if (v >= V) return;
    const float view = angles[v];
    DdView2 vw;
    dd_view2_scalars(geom, &g, view, &vw);
    if (threadIdx.x == 0) {
        views[v] = vw;
        ang[v] = view;
    }
    if (geom == DD_GEOM_PARA) return;
    const int D = g.num_det;
    float *dpv = dp + (size_t)v * (D + 1);
    for (int k = threadIdx.x; k <= D; k += blockDim.x) dpv[k] = dd_view2_boundary(geom, &g, view, &vw, k);
    __syncthreads();
    float *bc = bcoef + (size_t)v * (D + 1);
    for (int k = threadIdx.x; k < D; k += blockDim.x) bc[k] = dd_view2_bcoef(&g, &vw, dpv[k], dpv[k + 1]);
}

__global__ void k_lines(int geom, dd_geom2d g, const float *__restrict__ angles, int V, int nl,
                        const DdView2 *__restrict__ views, const float *__restrict__ dp,
                        DdLine *__restrict__ lines, DdLine *__restrict__ dlines) {
    const int v = blockIdx.y;
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const DdView2 vw = views[v];
    const int nline = vw.xb ? g.height : g.width;
    if (line >= nline) return;
    const size_t r = (size_t)v * nl + line;
    dd_line2_setup(geom, &g, angles[v], &vw, dp + (size_t)v * (g.num_det + 1), line, lines + r,
                   dlines ? dlines + r : nullptr);
}

// ---------------------------------------------------------------------------
// Prefix tables
// ---------------------------------------------------------------------------
// Row lines (x-branch): one warp per (image, row); S_j = sum_{i<j} x_i in FP64,
// rounded once.  Entry n = (S_n, 0).
__global__ void k_tab_rows(const float *__restrict__ img, int B, int H, int W,
                           float2 *__restrict__ tab) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B * H) return;
    const float *row = img + (size_t)warp * W;
    float2 *t = tab + (size_t)warp * rs_entries(W);
    double run = 0.0;
    for (int j0 = 0; j0 <= W; j0 += 32) {
        const int j = j0 + lane;
        const float x = (j < W) ? row[j] : 0.0f;
        double inc = (double)x;
        // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        const double excl = run + inc - (double)x;
        if (j <= W) t[j] = make_float2((float)excl, x);
        run += __shfl_sync(0xffffffffu, inc, 31);
    }
}

// Column lines (y-branch): line = image column, walked from the bottom row.
// One thread per (image, column): coalesced reads along a row.
__global__ void k_tab_cols(const float *__restrict__ img, int B, int H, int W,
                           float2 *__restrict__ tab) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * W) return;
    const int b = idx / W, col = idx - b * W;
    const float *im = img + (size_t)b * H * W;
    float2 *t = tab + (size_t)idx * rs_entries(H);
    double run = 0.0;
    for (int i = 0; i < H; i++) {
        const float x = im[(size_t)(H - 1 - i) * W + col];
        t[i] = make_float2((float)run, x);
        run += (double)x;
    }
    t[H] = make_float2((float)run, 0.0f);
}

// Detector tables for the adjoint: per (image, view) G_k and g_k over the
// sorted bins.  Fan: G_k = sum_{m<k} g_m (d_{m+1} - d_m) (exact widths);
// parallel: unit prefix (the drifted widths enter through the line pieces).
// mode 0: g = s * bcoef (ProjTrans), mode 1: g = s (BackProj family).
__global__ void k_dettab(int geom, int mode, const float *__restrict__ sino, int B, int V, int D,
                         const DdView2 *__restrict__ views, const float *__restrict__ dp,
                         const float *__restrict__ bcoef, float para_coef_x, float para_coef_y,
                         float2 *__restrict__ tab) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B * V) return;
    const int b = warp / V, v = warp - b * V;
    const DdView2 vw = views[v];
    const float *s = sino + ((size_t)b * V + v) * D;
    const float *dpv = dp + (size_t)v * (D + 1);
    const float *bc = bcoef + (size_t)v * (D + 1);
    float2 *t = tab + (size_t)warp * rs_entries(D);
    const float pc = vw.xb ? para_coef_x : para_coef_y;
    double run = 0.0;
    for (int k0 = 0; k0 <= D; k0 += 32) {
        const int k = k0 + lane;
        float gk = 0.0f;
        double w = 0.0;
        if (k < D) {
            const float sv = s[vw.flip ? D - 1 - k : k];
            if (geom == DD_GEOM_PARA) {
                gk = (mode == 0) ? sv * pc : sv;
                w = 1.0;
            } else {
                gk = (mode == 0) ? sv * bc[k] : sv;
                w = (double)(dpv[k + 1] - dpv[k]);
            }
        }
        double inc = (double)gk * w;
        const double mine = inc;
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (k <= D) t[k] = make_float2((float)(run + inc - mine), gk);
        run += __shfl_sync(0xffffffffu, inc, 31);
    }
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
struct FwdSmem {
    // dynamic layout offsets (bytes)
    int rec, drec, tab, kt, dp, bar, total;
};

__host__ __device__ inline FwdSmem fwd_smem(int geom, int D, int rsmax) {
    FwdSmem s;
    int o = 0;
    s.rec = o; o += 2 * (int)sizeof(DdLine);
    s.drec = o; if (geom == DD_GEOM_PARA) o += 2 * (int)sizeof(DdLine);
    s.tab = o; o += 2 * kBI * rsmax * (int)sizeof(float2);
    s.kt = o; o += kBI * 32 * (int)sizeof(float) * 2;   // K for pixel pieces (x2 for para det)
    s.dp = o; o += ((D + 1 + 3) & ~3) * (int)sizeof(float);
    s.bar = o; o += 2 * (int)sizeof(uint64_t);
    s.total = (o + 127) & ~127;
    return s;
}

template <int GEOM, int WEIGHTED>
__global__ void __launch_bounds__(kThreads)
k_fwd(dd_geom2d g, int op, int B, int V, int nl, const DdView2 *__restrict__ views,
      const float *__restrict__ dp, const float *__restrict__ bcoef,
      const DdLine *__restrict__ lines, const DdLine *__restrict__ dlines,
      const float2 *__restrict__ tabx, const float2 *__restrict__ taby, float *__restrict__ out,
      int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int v = blockIdx.x;
    const int b0 = blockIdx.y * kBI;
    const int nb = min(kBI, B - b0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int D = g.num_det;
    const DdView2 vw = views[v];
    const int xb = vw.xb;
    const int nline = xb ? g.height : g.width;
    const int npix = xb ? g.width : g.height;
    const int rs = rs_entries(npix);
    const int rsmax = rs_entries(g.width > g.height ? g.width : g.height);
    const FwdSmem L = fwd_smem(GEOM, D, rsmax);
    DdLine *rec = reinterpret_cast<DdLine *>(smem + L.rec);
    DdLine *drec = reinterpret_cast<DdLine *>(smem + L.drec);
    float2 *tab = reinterpret_cast<float2 *>(smem + L.tab);
    float *kt = reinterpret_cast<float *>(smem + L.kt);
    float *dps = reinterpret_cast<float *>(smem + L.dp);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L.bar);
    __shared__ int abort_flag;
    __shared__ float wsum[kWarps];

    const float2 *tsrc = xb ? tabx : taby;
    const size_t line_stride = (size_t)rs;                 // float2 per line
    const size_t img_stride = (size_t)nline * rs;          // float2 per image
    const uint32_t tab_bytes = (uint32_t)(rs * sizeof(float2));
    const uint32_t rec_bytes = (uint32_t)sizeof(DdLine);
    const uint32_t tx_bytes = nb * tab_bytes + rec_bytes + (GEOM == DD_GEOM_PARA ? rec_bytes : 0);

    if (tid == 0) {
        abort_flag = 0;
        dd_mbar_init(&bar[0], 1);
        dd_mbar_init(&bar[1], 1);
        dd_fence_mbar_init();
    }
    if (GEOM != DD_GEOM_PARA)
        for (int k = tid; k <= D; k += kThreads) dps[k] = dp[(size_t)v * (D + 1) + k];
    __syncthreads();

    auto issue = [&](int line, int buf) {
        dd_mbar_expect_tx(&bar[buf], tx_bytes);
        dd_bulk_g2s(rec + buf, lines + (size_t)v * nl + line, rec_bytes, &bar[buf]);
        if (GEOM == DD_GEOM_PARA)
            dd_bulk_g2s(drec + buf, dlines + (size_t)v * nl + line, rec_bytes, &bar[buf]);
        for (int b = 0; b < nb; b++)
            dd_bulk_g2s(tab + ((size_t)buf * kBI + b) * rsmax,
                        tsrc + (size_t)(b0 + b) * img_stride + (size_t)line * line_stride, tab_bytes,
                        &bar[buf]);
    };

    const int npass = (D + kWarps * kBinsPerWarp - 1) / (kWarps * kBinsPerWarp);
    constexpr int kMaxPass = 8;   // D <= 8 * 248 = 1984 detector bins
    float acc[kMaxPass][kBI];
#pragma unroll
    for (int m = 0; m < kMaxPass; m++)
#pragma unroll
        for (int b = 0; b < kBI; b++) acc[m][b] = 0.0f;

    const float para_beta = xb ? FDIV(g.pix_y, g.det_size) : FDIV(g.pix_x, g.det_size);
    if (tid == 0) issue(0, 0);

    for (int line = 0; line < nline; line++) {
        const int buf = line & 1;
        if (tid == 0 && line + 1 < nline) issue(line + 1, buf ^ 1);
        if (!dd_mbar_wait(&bar[buf], (line >> 1) & 1)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
        const DdLine &R = rec[buf];
        const int np = R.h.npiece;
        if (WEIGHTED && np > 0) {
            // BackProjTransWeighted: multiply every pixel by its FBP weight at
            // this view (FanFlatDisCPU2d.cpp:693, FanArcDisCPU2d.cpp:703) and
            // rebuild the line's prefix table in place (block scan).
            float2 *tw = tab + (size_t)buf * kBI * rsmax;
            const float lpos = xb
                ? (float)(((double)g.height / 2.0 - line - 0.5) * (double)g.pix_y + (double)g.pix_yshift)
                : (float)(((double)line - g.width / 2.0 + 0.5) * (double)g.pix_x + (double)g.pix_xshift);
            for (int b = 0; b < nb; b++) {
                float2 *t = tw + (size_t)b * rsmax;
                constexpr int kPer = 16;   // npix <= 4096
                const int per = (npix + kThreads - 1) / kThreads;
                float yv[kPer];
                float run = 0.0f;
#pragma unroll
                for (int q = 0; q < kPer; q++) {
                    const int i = tid * per + q;
                    float y = 0.0f;
                    if (q < per && i < npix) {
                        float pcx, pcy;
                        if (xb) {
                            pcx = (float)(((double)i + 0.5) * (double)g.pix_x + (double)vw.axis0);
                            pcy = lpos;
                        } else {
                            pcx = lpos;
                            pcy = (float)(((double)i + 0.5) * (double)g.pix_y + (double)vw.axis0);
                        }
                        const float w = (GEOM == DD_GEOM_ARC) ? 1.0f / dd_cw_arc(vw.srcx, vw.srcy, pcx, pcy)
                                                              : dd_cw_flat(vw.srcx, vw.srcy, pcx, pcy, g.iso_source);
                        y = t[i].y * w;
                    }
                    yv[q] = y;
                    run += y;
                }
                // exclusive scan of the per-thread sums across the block
                float inc = run;
                for (int o = 1; o < 32; o <<= 1) {
                    const float z = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += z;
                }
                if (lane == 31) wsum[warp] = inc;
                __syncthreads();
                float wbase = 0.0f;
                for (int w = 0; w < warp; w++) wbase += wsum[w];
                float pre = wbase + inc - run;
#pragma unroll
                for (int q = 0; q < kPer; q++) {
                    const int i = tid * per + q;
                    if (q < per && i < npix) {
                        t[i] = make_float2(pre, yv[q]);
                        pre += yv[q];
                    }
                }
                if (tid == kThreads - 1) {
                    float tot = 0.0f;
                    for (int w = 0; w < kWarps; w++) tot += wsum[w];
                    t[npix] = make_float2(tot, 0.0f);
                }
                __syncthreads();
            }
        }
        if (np > 0) {
            const float2 *tb = tab + (size_t)buf * kBI * rsmax;
            // per-piece constants, one warp per image
            for (int b = warp; b < nb; b += kWarps) {
                const float K = piece_K(R, tb + (size_t)b * rsmax, lane);
                kt[b * 32 + lane] = K;
            }
            __syncthreads();
            const float scale = (op == DD_OP_PROJ) ? 1.0f : R.h.alpha;
            const float bound0 = R.h.bound0, endv = R.h.endv;
            const int idet0 = R.h.idet0;
#pragma unroll
            for (int m = 0; m < kMaxPass; m++) {
                if (m >= npass) break;
                const int kb = m * (kWarps * kBinsPerWarp) + warp * kBinsPerWarp + lane;
                // boundary value: lower boundary of bin idet0 is the walk start
                float u;
                if (kb <= idet0) {
                    u = bound0;
                } else if (GEOM == DD_GEOM_PARA) {
                    const DdLine &Rd = drec[buf];
                    const int idx = min(kb - 1, D - 1);
                    const float est = Rd.p[0].Q + (float)(idx - Rd.p[0].gb) * Rd.p[0].dl;
                    u = (Rd.h.npiece > 0) ? dd_boundary(&Rd, idx, est) : bound0;
                } else {
                    u = dps[min(kb, D)];
                }
                u = fminf(fmaxf(u, bound0), endv);
                const Loc lc = locate(R, u);
#pragma unroll
                for (int b = 0; b < kBI; b++) {
                    if (b < nb) {
                        const float2 e = tb[(size_t)b * rsmax + lc.j];
                        const float f = fmaf(lc.r, e.y, fmaf(lc.dl, e.x, kt[b * 32 + lc.p]));
                        const float fn = __shfl_down_sync(0xffffffffu, f, 1);
                        if (lane < kBinsPerWarp) acc[m][b] = fmaf(scale, fn - f, acc[m][b]);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (abort_flag) {
        if (tid == 0) {
            atomicExch(status, DD_ERR_TIMEOUT);
            // let copies still in flight land before the CTA's shared memory goes away
            dd_mbar_wait(&bar[0], 0);
            dd_mbar_wait(&bar[1], 0);
        }
        __syncthreads();
        return;
    }
    // epilogue: bins of this warp/lane
#pragma unroll
    for (int m = 0; m < kMaxPass; m++) {
        if (m >= npass) break;
        const int k = m * (kWarps * kBinsPerWarp) + warp * kBinsPerWarp + lane;
        if (lane < kBinsPerWarp && k < D) {
            float beta = 1.0f;
            if (op == DD_OP_PROJ) beta = (GEOM == DD_GEOM_PARA) ? para_beta : bcoef[(size_t)v * (D + 1) + k];
            const int ko = vw.flip ? D - 1 - k : k;
            for (int b = 0; b < nb; b++)
                out[((size_t)(b0 + b) * V + v) * D + ko] = acc[m][b] * beta;
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint-type kernel (ProjTrans, BackProj, BackProjWeighted): pixel gathers.
// CTA = 32x32 image tile x kBI images; loops over all views, accumulating in
// registers (row-major ownership for x-branch views, column-major for
// y-branch views, merged through shared memory at the end).
// ---------------------------------------------------------------------------
constexpr int kTile = 32;
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

// Shared-memory layout of the adjoint kernel (bytes).
struct AdjSmem {
    int rec, drec, kd, bar, total;
};

__host__ __device__ inline AdjSmem adj_smem(int geom) {
    AdjSmem s;
    int o = 0;
    s.rec = o; o += 2 * kTile * (int)sizeof(DdLine);
    s.drec = o; if (geom == DD_GEOM_PARA) o += 2 * kTile * (int)sizeof(DdLine);
    s.kd = o; if (geom == DD_GEOM_PARA) o += kWarps * kBI * 32 * (int)sizeof(float);
    s.bar = o; o += 2 * (int)sizeof(uint64_t);
    // the final merge of the two pixel ownerships reuses the record buffers
    const int merge = kBI * kTile * (kTile + 1) * (int)sizeof(float);
    if (o < merge + 16) o = merge + 16;
    s.total = (o + 127) & ~127;
    return s;
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

template <int GEOM, int OPK>   // OPK: 0 ProjTrans, 1 BackProj, 2 BackProjWeighted
__global__ void __launch_bounds__(kThreads)
k_adj(dd_geom2d g, int B, int V, int nl, const float *__restrict__ angles,
      const DdView2 *__restrict__ views, const float *__restrict__ dp,
      const DdLine *__restrict__ lines, const DdLine *__restrict__ dlines,
      const float2 *__restrict__ dtab, float *__restrict__ out, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const AdjSmem SL = adj_smem(GEOM);
    DdLine *recs = reinterpret_cast<DdLine *>(smem + SL.rec);
    DdLine *drecs = reinterpret_cast<DdLine *>(smem + SL.drec);
    float *kdp = reinterpret_cast<float *>(smem + SL.kd);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + SL.bar);
    __shared__ int abort_flag;

    const int c0 = blockIdx.x * kTile, r0 = blockIdx.y * kTile;
    const int b0 = blockIdx.z * kBI;
    const int nb = min(kBI, B - b0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = g.width, H = g.height, D = g.num_det;
    const int rsd = rs_entries(D);

    if (tid == 0) {
        abort_flag = 0;
        dd_mbar_init(&bar[0], 1);
        dd_mbar_init(&bar[1], 1);
        dd_fence_mbar_init();
    }
    __syncthreads();

    // records of the tile's lines of view v: rows r0.. (x-branch) or columns c0..
    auto issue = [&](int v, int buf) {
        const int xbv = views[v].xb;
        const int line0 = xbv ? r0 : c0;
        const int nline = xbv ? H : W;
        const int n = min(kTile, nline - line0);
        const uint32_t bytes = (uint32_t)(n * sizeof(DdLine));
        dd_mbar_expect_tx(&bar[buf], bytes * (GEOM == DD_GEOM_PARA ? 2u : 1u));
        dd_bulk_g2s(recs + buf * kTile, lines + (size_t)v * nl + line0, bytes, &bar[buf]);
        if (GEOM == DD_GEOM_PARA)
            dd_bulk_g2s(drecs + buf * kTile, dlines + (size_t)v * nl + line0, bytes, &bar[buf]);
    };

    float ax[kLinesPerWarp][kBI], ay[kLinesPerWarp][kBI];
#pragma unroll
    for (int q = 0; q < kLinesPerWarp; q++)
#pragma unroll
        for (int b = 0; b < kBI; b++) ax[q][b] = ay[q][b] = 0.0f;

    if (tid == 0) issue(0, 0);
    for (int v = 0; v < V; v++) {
        const int buf = v & 1;
        if (tid == 0 && v + 1 < V) issue(v + 1, buf ^ 1);
        if (!dd_mbar_wait(&bar[buf], (v >> 1) & 1)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
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
                    pcx = (float)(((double)pi + 0.5) * (double)g.pix_x + (double)vw.axis0);
                    pcy = (float)(((double)H / 2.0 - line - 0.5) * (double)g.pix_y + (double)g.pix_yshift);
                } else {
                    pcx = (float)(((double)line - W / 2.0 + 0.5) * (double)g.pix_x + (double)g.pix_xshift);
                    pcy = (float)(((double)pi + 0.5) * (double)g.pix_y + (double)vw.axis0);
                }
                wgt = alpha * ((GEOM == DD_GEOM_ARC) ? 1.0f / dd_cw_arc(vw.srcx, vw.srcy, pcx, pcy)
                                                     : dd_cw_flat(vw.srcx, vw.srcy, pcx, pcy, g.iso_source));
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
                    const float2 *t = dtab + ((size_t)(b0 + b) * V + v) * rsd;
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
#pragma unroll
                for (int b = 0; b < kBI; b++) {
                    if (b >= nb) break;
                    const float2 *t = dtab + ((size_t)(b0 + b) * V + v) * rsd;
                    const float2 e = __ldg(t + kU);
                    const float hu = fmaf(offU, e.y, e.x);
                    float hl = __shfl_up_sync(0xffffffffu, hu, 1);
                    if (need_low) {
                        const float2 e2 = __ldg(t + kL);
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
        if (tid == 0) {
            atomicExch(status, DD_ERR_TIMEOUT);
            dd_mbar_wait(&bar[0], 0);
            dd_mbar_wait(&bar[1], 0);
        }
        __syncthreads();
        return;
    }
    // merge the two ownerships through shared memory (reusing the record buffers)
    float (*tile)[kTile][kTile + 1] = reinterpret_cast<float (*)[kTile][kTile + 1]>(smem + SL.rec);
    for (int b = 0; b < nb; b++) {
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) tile[b][warp + kWarps * q][lane] = ax[q][b];
    }
    __syncthreads();
    for (int b = 0; b < nb; b++) {
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) tile[b][kTile - 1 - lane][warp + kWarps * q] += ay[q][b];
    }
    __syncthreads();
    for (int b = 0; b < nb; b++) {
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; q++) {
            const int r = r0 + warp + kWarps * q, c = c0 + lane;
            if (r < H && c < W) out[((size_t)(b0 + b) * H + r) * W + c] = tile[b][warp + kWarps * q][lane];
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int geom_of(int scan) {
    return scan == DD_SCAN_PARA ? DD_GEOM_PARA : (scan == DD_SCAN_FLAT ? DD_GEOM_FLAT : DD_GEOM_ARC);
}

static int validate(int scan, int op, const dd_geom2d *g, int B, int V) {
    if (!g) return DD_ERR_INVALID_ARG;
    if (scan < DD_SCAN_PARA || scan > DD_SCAN_ARC) return DD_ERR_INVALID_ARG;
    if (op < DD_OP_PROJ || op > DD_OP_BPROJ_TW) return DD_ERR_INVALID_ARG;
    if (scan == DD_SCAN_PARA && (op == DD_OP_BPROJ_W || op == DD_OP_BPROJ_TW)) return DD_ERR_UNSUPPORTED;
    if (g->width <= 0 || g->height <= 0 || g->num_det <= 0 || B <= 0 || V <= 0) return DD_ERR_INVALID_ARG;
    const float f[] = {g->pix_x, g->pix_y, g->det_size, g->iso_source, g->source_detector,
                       g->pix_xshift, g->pix_yshift, g->bin_shift};
    for (float x : f)
        if (!(x == x) || x - x != 0.0f) return DD_ERR_INVALID_ARG;   // NaN / inf
    if (!(g->pix_x > 0 && g->pix_y > 0 && g->det_size > 0)) return DD_ERR_INVALID_ARG;
    if (scan != DD_SCAN_PARA && !(g->iso_source > 0 && g->source_detector > 0)) return DD_ERR_INVALID_ARG;
    const long long lim = (1LL << 31) - 1;
    if ((long long)g->width * g->height * B > lim) return DD_ERR_SIZE_OVERFLOW;
    if ((long long)V * g->num_det * B > lim) return DD_ERR_SIZE_OVERFLOW;
    if (g->width > 4096 || g->height > 4096) return DD_ERR_SIZE_OVERFLOW;
    if (g->num_det > 8 * kWarps * kBinsPerWarp) return DD_ERR_SIZE_OVERFLOW;
    return DD_OK;
}

static int launch_status() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? DD_OK : DD_ERR_LAUNCH;
}

// ---------------------------------------------------------------------------
// Launch accounting and optional per-kernel event timing (benchmarks only;
// never enabled during graph capture)
// ---------------------------------------------------------------------------
static unsigned long long g_launches = 0;
static int g_prof = 0;
struct ProfRec {
    cudaEvent_t a, b;
    int kind;
};
static ProfRec g_prof_rec[8192];
static int g_prof_used = 0;
static int g_prof_created = 0;

static ProfRec *prof_begin(int kind, cudaStream_t st) {
    if (!g_prof || g_prof_used >= 8192) return nullptr;
    ProfRec *r = &g_prof_rec[g_prof_used];
    if (g_prof_used >= g_prof_created) {
        if (cudaEventCreate(&r->a) != cudaSuccess || cudaEventCreate(&r->b) != cudaSuccess) return nullptr;
        g_prof_created++;
    }
    g_prof_used++;
    r->kind = kind;
    cudaEventRecord(r->a, st);
    return r;
}
static void prof_end(ProfRec *r, cudaStream_t st) {
    if (r) cudaEventRecord(r->b, st);
}

int plan(int scan, const dd_geom2d *g, const float *angles, int V, void *planp, size_t bytes,
         cudaStream_t st) {
    const PlanLayout P = plan_layout(scan, g, V);
    if (!planp || bytes < P.total) return DD_ERR_WORKSPACE;
    if (!angles) return DD_ERR_INVALID_ARG;
    char *base = (char *)planp;
    const int geom = geom_of(scan);
    DdView2 *views = (DdView2 *)(base + P.views);
    float *dp = (float *)(base + P.dp);
    float *bc = (float *)(base + P.bcoef);
    DdLine *lines = (DdLine *)(base + P.lines);
    DdLine *dlines = scan == DD_SCAN_PARA ? (DdLine *)(base + P.dlines) : nullptr;
    ProfRec *pr = prof_begin(DD_KERNEL_PLAN, st);
    k_views<<<V, 256, 0, st>>>(geom, *g, angles, V, views, (float *)(base + P.ang), dp, bc);
    dim3 gl((P.nl + 63) / 64, V);
    k_lines<<<gl, 64, 0, st>>>(geom, *g, angles, V, P.nl, views, dp, lines, dlines);
    prof_end(pr, st);
    g_launches += 2;
    return launch_status();
}

template <int GEOM>
static int launch_fwd(int op, const dd_geom2d *g, const PlanLayout &P, const char *planb, int B,
                      int V, const float2 *tx, const float2 *ty, float *out, int *status,
                      cudaStream_t st) {
    const int rsmax = rs_entries(g->width > g->height ? g->width : g->height);
    const FwdSmem S = fwd_smem(GEOM, g->num_det, rsmax);
    dim3 grid(V, (B + kBI - 1) / kBI);
    const DdView2 *views = (const DdView2 *)(planb + P.views);
    const float *dp = (const float *)(planb + P.dp);
    const float *bc = (const float *)(planb + P.bcoef);
    const DdLine *lines = (const DdLine *)(planb + P.lines);
    const DdLine *dlines = GEOM == DD_GEOM_PARA ? (const DdLine *)(planb + P.dlines) : nullptr;
    auto kern = (op == DD_OP_BPROJ_TW) ? k_fwd<GEOM, 1> : k_fwd<GEOM, 0>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S.total) != cudaSuccess)
        return DD_ERR_LAUNCH;
    ProfRec *pr = prof_begin(DD_KERNEL_FORWARD, st);
    kern<<<grid, kThreads, S.total, st>>>(*g, op, B, V, P.nl, views, dp, bc, lines, dlines, tx, ty,
                                          out, status);
    prof_end(pr, st);
    g_launches++;
    return launch_status();
}

template <int GEOM>
static int launch_adj(int op, const dd_geom2d *g, const PlanLayout &P, const char *planb,
                      const float *angles, int B, int V, const float2 *dtab, float *out, int *status,
                      cudaStream_t st) {
    dim3 grid((g->width + kTile - 1) / kTile, (g->height + kTile - 1) / kTile, (B + kBI - 1) / kBI);
    const DdView2 *views = (const DdView2 *)(planb + P.views);
    const float *dp = (const float *)(planb + P.dp);
    const DdLine *lines = (const DdLine *)(planb + P.lines);
    const DdLine *dlines = GEOM == DD_GEOM_PARA ? (const DdLine *)(planb + P.dlines) : nullptr;
    const AdjSmem S = adj_smem(GEOM);
    auto kern = (op == DD_OP_PROJ_T) ? k_adj<GEOM, 0> : (op == DD_OP_BPROJ) ? k_adj<GEOM, 1> : k_adj<GEOM, 2>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S.total) != cudaSuccess)
        return DD_ERR_LAUNCH;
    ProfRec *pr = prof_begin(DD_KERNEL_ADJOINT, st);
    kern<<<grid, kThreads, S.total, st>>>(*g, B, V, P.nl, angles, views, dp, lines, dlines, dtab, out, status);
    prof_end(pr, st);
    g_launches++;
    return launch_status();
}

int apply_planned(int scan, int op, const dd_geom2d *g, const void *planp, const float *in,
                  float *out, int B, int V, void *ws, size_t wsb, cudaStream_t st) {
    const PlanLayout P = plan_layout(scan, g, V);
    const float *angles = (const float *)((const char *)planp + P.ang);
    const ApplyLayout A = apply_layout(op, g, B, V);
    if (!ws || wsb < A.total) return DD_ERR_WORKSPACE;
    if (!in || !out || !planp) return DD_ERR_INVALID_ARG;
    const char *planb = (const char *)planp;
    char *wb = (char *)ws;
    int *status = (int *)(wb + A.status);
    const int geom = geom_of(scan);
    const int W = g->width, H = g->height;
    if (op_is_forward(op)) {
        float2 *tx = (float2 *)(wb + A.tabx), *ty = (float2 *)(wb + A.taby);
        const int nw = B * H;
        ProfRec *pr = prof_begin(DD_KERNEL_TABLES, st);
        k_tab_rows<<<(nw * 32 + 255) / 256, 256, 0, st>>>(in, B, H, W, tx);
        k_tab_cols<<<(B * W + 127) / 128, 128, 0, st>>>(in, B, H, W, ty);
        prof_end(pr, st);
        g_launches += 2;
        if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
        if (geom == DD_GEOM_PARA) return launch_fwd<DD_GEOM_PARA>(op, g, P, planb, B, V, tx, ty, out, status, st);
        if (geom == DD_GEOM_FLAT) return launch_fwd<DD_GEOM_FLAT>(op, g, P, planb, B, V, tx, ty, out, status, st);
        return launch_fwd<DD_GEOM_ARC>(op, g, P, planb, B, V, tx, ty, out, status, st);
    }
    float2 *dtab = (float2 *)(wb + A.dtab);
    const int mode = (op == DD_OP_PROJ_T) ? 0 : 1;
    const float pcx = g->pix_y / g->det_size, pcy = g->pix_x / g->det_size;
    const int nw = B * V;
    ProfRec *pr = prof_begin(DD_KERNEL_TABLES, st);
    g_launches++;
    k_dettab<<<(nw * 32 + 255) / 256, 256, 0, st>>>(geom, mode, in, B, V, g->num_det,
                                                     (const DdView2 *)(planb + P.views),
                                                     (const float *)(planb + P.dp),
                                                     (const float *)(planb + P.bcoef), pcx, pcy, dtab);
    prof_end(pr, st);
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    if (geom == DD_GEOM_PARA) return launch_adj<DD_GEOM_PARA>(op, g, P, planb, angles, B, V, dtab, out, status, st);
    if (geom == DD_GEOM_FLAT) return launch_adj<DD_GEOM_FLAT>(op, g, P, planb, angles, B, V, dtab, out, status, st);
    return launch_adj<DD_GEOM_ARC>(op, g, P, planb, angles, B, V, dtab, out, status, st);
}

}  // namespace dd2

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace dd2;

extern "C" int dd2d_validate(int scan, int op, const dd_geom2d *g, int batch, int num_view) {
    return validate(scan, op, g, batch, num_view);
}

extern "C" size_t dd2d_plan_bytes(int scan, const dd_geom2d *g, int num_view) {
    if (!g || num_view <= 0) return 0;
    return plan_layout(scan, g, num_view).total;
}

extern "C" size_t dd2d_apply_workspace_bytes(int scan, int op, const dd_geom2d *g, int batch,
                                             int num_view) {
    (void)scan;
    if (!g || batch <= 0 || num_view <= 0) return 0;
    return apply_layout(op, g, batch, num_view).total;
}

extern "C" size_t dd2d_workspace_bytes(int scan, int op, const dd_geom2d *g, int batch, int num_view) {
    if (!g || batch <= 0 || num_view <= 0) return 0;
    return plan_layout(scan, g, num_view).total + apply_layout(op, g, batch, num_view).total;
}

extern "C" int dd2d_plan(int scan, const dd_geom2d *g, const float *angles, int num_view, void *planp,
                         size_t plan_bytes, dd_stream_t stream) {
    const int st = validate(scan, DD_OP_PROJ, g, 1, num_view);
    if (st != DD_OK) return st;
    return plan(scan, g, angles, num_view, planp, plan_bytes, (cudaStream_t)stream);
}

extern "C" int dd2d_apply(int scan, int op, const dd_geom2d *g, const float *in, float *out,
                          const float *angles, int batch, int num_view, void *workspace,
                          size_t workspace_bytes, dd_stream_t stream) {
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!angles || !in || !out) return DD_ERR_INVALID_ARG;
    const size_t pb = plan_layout(scan, g, num_view).total;
    if (!workspace || workspace_bytes < dd2d_workspace_bytes(scan, op, g, batch, num_view))
        return DD_ERR_WORKSPACE;
    const int s1 = plan(scan, g, angles, num_view, workspace, pb, (cudaStream_t)stream);
    if (s1 != DD_OK) return s1;
    return apply_planned(scan, op, g, workspace, in, out, batch, num_view, (char *)workspace + pb,
                         workspace_bytes - pb, (cudaStream_t)stream);
}

extern "C" int dd2d_apply_planned(int scan, int op, const dd_geom2d *g, const void *planp,
                                  const float *in, float *out, int batch, int num_view,
                                  void *workspace, size_t workspace_bytes, dd_stream_t stream) {
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    return apply_planned(scan, op, g, planp, in, out, batch, num_view, workspace, workspace_bytes,
                         (cudaStream_t)stream);
}

// named entries (RadonTorch.cpp:1376-1393)
#define DD_NAMED(name, scan, op)                                                              \
    extern "C" int dd_##name(const dd_geom2d *g, const float *in, float *out,                 \
                             const float *angles, int batch, int num_view, void *workspace,   \
                             size_t workspace_bytes, dd_stream_t stream) {                    \
        return dd2d_apply(scan, op, g, in, out, angles, batch, num_view, workspace,           \
                          workspace_bytes, stream);                                           \
    }
DD_NAMED(ProjFanFlatDis2d, DD_SCAN_FLAT, DD_OP_PROJ)
DD_NAMED(ProjTransFanFlatDis2d, DD_SCAN_FLAT, DD_OP_PROJ_T)
DD_NAMED(BackProjFanFlatDis2d, DD_SCAN_FLAT, DD_OP_BPROJ)
DD_NAMED(BackProjTransFanFlatDis2d, DD_SCAN_FLAT, DD_OP_BPROJ_T)
DD_NAMED(BackProjWeightedFanFlatDis2d, DD_SCAN_FLAT, DD_OP_BPROJ_W)
DD_NAMED(BackProjTransWeightedFanFlatDis2d, DD_SCAN_FLAT, DD_OP_BPROJ_TW)
DD_NAMED(ProjFanArcDis2d, DD_SCAN_ARC, DD_OP_PROJ)
DD_NAMED(ProjTransFanArcDis2d, DD_SCAN_ARC, DD_OP_PROJ_T)
DD_NAMED(BackProjFanArcDis2d, DD_SCAN_ARC, DD_OP_BPROJ)
DD_NAMED(BackProjTransFanArcDis2d, DD_SCAN_ARC, DD_OP_BPROJ_T)
DD_NAMED(BackProjWeightedFanArcDis2d, DD_SCAN_ARC, DD_OP_BPROJ_W)
DD_NAMED(BackProjTransWeightedFanArcDis2d, DD_SCAN_ARC, DD_OP_BPROJ_TW)
DD_NAMED(ProjParaDis2d, DD_SCAN_PARA, DD_OP_PROJ)
DD_NAMED(ProjTransParaDis2d, DD_SCAN_PARA, DD_OP_PROJ_T)
DD_NAMED(BackProjParaDis2d, DD_SCAN_PARA, DD_OP_BPROJ)
DD_NAMED(BackProjTransParaDis2d, DD_SCAN_PARA, DD_OP_BPROJ_T)
#undef DD_NAMED

extern "C" const char *dd_status_string(int status) {
    switch (status) {
    case DD_OK: return "ok";
    case DD_ERR_INVALID_ARG: return "invalid argument (null pointer, non-positive size or non-finite geometry)";
    case DD_ERR_SIZE_OVERFLOW: return "sizes exceed the supported index range";
    case DD_ERR_WORKSPACE: return "workspace missing or too small";
    case DD_ERR_LAUNCH: return "CUDA launch or runtime error";
    case DD_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    case DD_ERR_UNSUPPORTED: return "operator not defined for this geometry";
    default: return "unknown status";
    }
}

extern "C" const char *dd_version(void) { return "pridediff_dd 0.1 sm_103a"; }

extern "C" unsigned long long dd_launch_count(void) { return g_launches; }

extern "C" int dd_profile_enable(int on) {
    g_prof = on ? 1 : 0;
    g_prof_used = 0;
    return DD_OK;
}

extern "C" int dd_profile_read(int kind, double *total_ms, int *count) {
    if (!total_ms || !count) return DD_ERR_INVALID_ARG;
    double t = 0.0;
    int n = 0;
    for (int i = 0; i < g_prof_used; i++) {
        if (g_prof_rec[i].kind != kind) continue;
        if (cudaEventSynchronize(g_prof_rec[i].b) != cudaSuccess) return DD_ERR_LAUNCH;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, g_prof_rec[i].a, g_prof_rec[i].b) != cudaSuccess) return DD_ERR_LAUNCH;
        t += ms;
        n++;
    }
    *total_ms = t;
    *count = n;
    return DD_OK;
}
