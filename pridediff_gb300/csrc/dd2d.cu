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

#include <algorithm>
#include <stdint.h>
#include <string.h>

#include "dd2d_kernels.cuh"
#include "dd_trace.h"

namespace dd2 {
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
// Row lines (x-branch): one warp per (image, row); S_j = sum_{i<j} x_i in
// double-float arithmetic, rounded once.  Entry n = (S_n, 0).
__global__ void k_tab_rows(const float *__restrict__ img, int B, int H, int W,
                           float2 *__restrict__ tab) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B * H) return;
    const float *row = img + (size_t)warp * W;
    warp_prefix_table(W, tab + (size_t)warp * rs_entries(W), lane, [&](int j, float *x, float *w) {
        *x = row[j];
        *w = 1.0f;
    });
}

// Column lines (y-branch): line = image column, walked from the bottom row.
// A block takes 32 columns of one image (lanes: coalesced reads along a row)
// and splits the rows into kColChunks chunks (warps): each warp sums its
// chunk in double-float arithmetic, the chunk totals are added in order, and
// each warp then writes its rows' prefixes from its chunk's start -- 8 times
// the threads of one walk per column.
constexpr int kColChunks = 8;
__global__ void __launch_bounds__(32 * kColChunks)
k_tab_cols(const float *__restrict__ img, int B, int H, int W, float2 *__restrict__ tab) {
    const int c = threadIdx.x & 31, k = threadIdx.x >> 5;
    const int ncb = (W + 31) / 32;
    const int b = blockIdx.x / ncb, col = (blockIdx.x - b * ncb) * 32 + c;
    const int per = (H + kColChunks - 1) / kColChunks;
    const int i0 = min(H, k * per), i1 = min(H, i0 + per);
    const bool ok = b < B && col < W;
    const float *__restrict__ im = img + (size_t)b * H * W + col;
    __shared__ float tot_hi[kColChunks][32], tot_lo[kColChunks][32];
    DdF run = {0.0f, 0.0f};
    if (ok)
        for (int i = i0; i < i1; i++) run = df_add(run, DdF{__ldg(im + (size_t)(H - 1 - i) * W), 0.0f});
    tot_hi[k][c] = run.hi;
    tot_lo[k][c] = run.lo;
    __syncthreads();
    if (!ok) return;
    run = {0.0f, 0.0f};
    for (int q = 0; q < k; q++) run = df_add(run, DdF{tot_hi[q][c], tot_lo[q][c]});
    float2 *__restrict__ t = tab + ((size_t)b * W + col) * rs_entries(H);
    for (int i = i0; i < i1; i++) {
        const float x = __ldg(im + (size_t)(H - 1 - i) * W);
        t[i] = make_float2(run.hi, x);
        run = df_add(run, DdF{x, 0.0f});
    }
    if (i0 < H && i1 == H) t[H] = make_float2(run.hi, 0.0f);
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
    const float pc = vw.xb ? para_coef_x : para_coef_y;
    warp_prefix_table(D, tab + (size_t)warp * rs_entries(D), lane, [&](int k, float *g, float *w) {
        const float sv = s[vw.flip ? D - 1 - k : k];
        if (geom == DD_GEOM_PARA) {
            *g = (mode == 0) ? sv * pc : sv;
            *w = 1.0f;
        } else {
            *g = (mode == 0) ? sv * bc[k] : sv;
            *w = dpv[k + 1] - dpv[k];
        }
    });
}

// Single-geometry forward launch: grid (views, image groups).
// Shape of the single-geometry forward CTA: kFwdWarps warps over kFwdImages
// slices.  The per-boundary locate in a line's drift record is shared by the
// CTA's slices while the double-buffered line tables grow with them; on the
// 16 x 512^2, 720-view workload 8 warps x 4 slices (4.62 ms) beat 8 x 8
// (5.39 ms), 8 x 2 (6.02 ms) and 16 x 8 (5.27 ms).
constexpr int kFwdImages = 4;
constexpr int kFwdWarps = 8;

// blockIdx.x = view * CL + rank in the view's cluster of CL CTAs.
template <int GEOM, int WEIGHTED, int NPASS, int NW, int BI, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NW * 32, (BI == 1 && NPASS <= 4) ? 8 : 0)
k_fwd(dd_geom2d g, int op, int B, int V, int nl, const DdView2 *__restrict__ views,
      const float *__restrict__ dp, const float *__restrict__ bcoef,
      const DdLine *__restrict__ lines, const DdLine *__restrict__ dlines,
      const float2 *__restrict__ tabx, const float2 *__restrict__ taby, float *__restrict__ out,
      const float *__restrict__ sub, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int rsmax = rs_entries(g.width > g.height ? g.width : g.height);
    const FwdSmem L = fwd_smem(GEOM, g.num_det, rsmax, BI, CL, NW);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L.bar);
    init_bars(bar);
    DdPhases ph;
    FwdItem it;
    it.v = blockIdx.x / CL;
    it.b0 = blockIdx.y * BI;
    it.nb = min(BI, B - it.b0);
    it.V = V;
    it.nl = nl;
    it.views = views;
    it.dp = dp;
    it.bcoef = bcoef;
    it.lines = lines;
    it.dlines = dlines;
    it.tabx = tabx;
    it.taby = taby;
    it.out = out;
    it.sub = sub;
    if (!fwd_view<GEOM, WEIGHTED, NPASS, BI, NW, CL>(g, op, it, smem, g.num_det, rsmax, ph) &&
        threadIdx.x == 0)
        dd_report_timeout(status);
}

// Parallel beam (plan time): the views that walk image rows and those that
// walk columns, each in view order.  One warp: ballots rank the views.
__global__ void __launch_bounds__(32)
k_axis_views(int V, const DdView2 *__restrict__ views, int *__restrict__ axisv) {
    const int lane = threadIdx.x;
    const unsigned below = (1u << lane) - 1u;
    int nr = 0, nc = 0;
    for (int v0 = 0; v0 < V; v0 += 32) {
        const int v = v0 + lane;
        const bool in = v < V;
        const bool xb = in && views[v].xb;
        const unsigned mr = __ballot_sync(0xffffffffu, xb), mc = __ballot_sync(0xffffffffu, in && !xb);
        if (xb) axisv[2 + nr + __popc(mr & below)] = v;
        else if (in) axisv[2 + V + nc + __popc(mc & below)] = v;
        nr += __popc(mr);
        nc += __popc(mc);
    }
    if (lane == 0) {
        axisv[0] = nr;
        axisv[1] = nc;
    }
}

// ---------------------------------------------------------------------------
// Parallel-beam adjoint, line-major.  The parallel beam's detector boundaries
// drift per walked line (ParaDisCPU2d.cpp:76, :100: the recurrence restarts
// at each line's first bin), so every (view, line, image) needs its own piece
// constants of the detector table.  One CTA takes one walked line and a group
// of kBI images over all the views that walk its axis, builds the line's
// piece constants once per view and serves all the line's pixels from them
// (a 32 x 32 tile rebuilds them for each tile the line crosses).  A thread
// owns fixed pixels of the line; their sums stay in shared memory.  The rows
// (x-branch views) are written by one launch and the columns added by a
// second, the same order as the tiled kernel's merge of its two ownerships,
// with the same per-pixel arithmetic.
// ---------------------------------------------------------------------------
struct ParaSmem {
    int rec, drec, tab, kt, acc, bar, total;
};
__host__ __device__ inline ParaSmem para_smem(int D, int npix) {
    ParaSmem s;
    int o = 0;
    s.rec = o; o += 2 * (int)sizeof(DdLine);
    s.drec = o; o += 2 * (int)sizeof(DdLine);
    s.tab = o; o += 2 * kBI * rs_entries(D) * (int)sizeof(float2);
    s.kt = o; o += kBI * 32 * (int)sizeof(float);
    s.acc = o; o += ((kBI * npix + 3) & ~3) * (int)sizeof(float);
    s.bar = o; o += 2 * (int)sizeof(uint64_t);
    s.total = (o + 127) & ~127;
    return s;
}

template <int OPK>   // 0 ProjTrans, 1 BackProj
__global__ void __launch_bounds__(kThreads)
k_adj_para(dd_geom2d g, int B, int V, int nl, int axis, const int *__restrict__ axisv,
           const DdLine *__restrict__ lines, const DdLine *__restrict__ dlines,
           const float2 *__restrict__ dtab, float *__restrict__ out, const float *__restrict__ base,
           float scale, int add, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int W = g.width, H = g.height, D = g.num_det;
    const int npix = axis ? W : H;
    const int line = blockIdx.x, b0 = blockIdx.y * kBI, nb = min(kBI, B - b0);
    const int nv = axisv[axis ? 0 : 1];
    const int *vlist = axisv + 2 + (axis ? 0 : V);
    const int rsd = rs_entries(D);
    const ParaSmem S = para_smem(D, npix);
    DdLine *rec = reinterpret_cast<DdLine *>(smem + S.rec);
    DdLine *drec = reinterpret_cast<DdLine *>(smem + S.drec);
    float2 *tabs = reinterpret_cast<float2 *>(smem + S.tab);   // [2][kBI][rsd]
    float *kt = reinterpret_cast<float *>(smem + S.kt);        // [kBI][32]
    float *accs = reinterpret_cast<float *>(smem + S.acc);     // [kBI][npix]
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + S.bar);
    __shared__ int abort_flag;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < kBI * npix; i += kThreads) accs[i] = 0.0f;
    if (tid == 0) abort_flag = 0;
    init_bars(bar);   // synchronises the CTA
    DdPhases ph;

    const uint32_t rec_bytes = (uint32_t)sizeof(DdLine);
    const uint32_t tab_bytes = (uint32_t)(rsd * sizeof(float2));
    auto issue = [&](int idx, int buf) {
        const int v = vlist[idx];
        dd_mbar_expect_tx(&bar[buf], 2 * rec_bytes + nb * tab_bytes);
        dd_bulk_g2s(rec + buf, lines + (size_t)v * nl + line, rec_bytes, &bar[buf]);
        dd_bulk_g2s(drec + buf, dlines + (size_t)v * nl + line, rec_bytes, &bar[buf]);
        for (int b = 0; b < nb; b++)
            dd_bulk_g2s(tabs + ((size_t)buf * kBI + b) * rsd, dtab + ((size_t)(b0 + b) * V + v) * rsd, tab_bytes,
                        &bar[buf]);
    };
    const int issuer = (kWarps - 1) * 32;
    if (tid == issuer && nv > 0) issue(0, 0);
    for (int idx = 0; idx < nv; idx++) {
        const int buf = idx & 1;
        if (!dd_mbar_wait(&bar[buf], ph.parity(buf))) abort_flag = 1;
        ph.flip(buf);
        // past this barrier every warp has finished view idx - 1, whose
        // buffer takes the copies of view idx + 1
        __syncthreads();
        if (abort_flag) {
            // view idx's copies (the wait gave up on them) may be in flight
            if (tid == issuer) dd_mbar_drain(&bar[buf], ph.parity(buf) ^ 1u);
            break;
        }
        if (tid == issuer && idx + 1 < nv) issue(idx + 1, buf ^ 1);
        const DdLine &L = rec[buf], &Ld = drec[buf];
        if (L.h.npiece == 0) continue;   // the same for the whole CTA
        const int npd = Ld.h.npiece;
        const float2 *tb = tabs + (size_t)buf * kBI * rsd;
        for (int b = warp; b < nb; b += kWarps) kt[b * 32 + lane] = npd > 0 ? piece_K(Ld, tb + (size_t)b * rsd, lane) : 0.0f;
        __syncthreads();
        const int i0 = L.h.i0, nend = L.h.nend;
        const float bound0 = L.h.bound0;
        const float alpha = (OPK == 0) ? 1.0f : L.h.alpha;
        // a warp takes 32 consecutive pixel boundaries (lane l: the upper
        // boundary of pixel q0 + l - 1) and 31 pixels: each boundary is
        // located once and neighbours difference by one shuffle
        for (int q0 = warp * kBinsPerWarp; q0 < npix; q0 += kWarps * kBinsPerWarp) {   // warp-uniform
            const int bi = q0 + lane - 1;   // boundary index (upper boundary of pixel bi)
            float u = bound0;               // boundary i0 - 1 is the walk start; below it H is constant
            if (bi >= i0 && bi < nend) u = dd_boundary(&L, bi, L.p[0].Q + (float)(bi - L.p[0].gb) * L.p[0].dl);
            int pU = 0, jU = 0;
            float rU = 0.0f, dlU = 0.0f;
            if (npd > 0) {
                dd_locate(&Ld, fminf(fmaxf(u, bound0), Ld.h.endv), &pU, &jU, &rU);
                dlU = Ld.p[pU].dl;
            }
            const int pi = bi;   // the pixel this lane closes (lanes 1..31)
            const bool valid = lane > 0 && pi < npix && pi >= i0 && pi < nend;
#pragma unroll
            for (int b = 0; b < kBI; b++) {
                if (b >= nb) break;
                float hu = 0.0f;
                if (npd > 0) {
                    const float2 e = tb[(size_t)b * rsd + jU];
                    hu = fmaf(rU, e.y, fmaf(dlU, e.x, kt[b * 32 + pU]));
                }
                const float hl = __shfl_up_sync(0xffffffffu, hu, 1);
                if (valid) accs[b * npix + pi] += alpha * (hu - hl);
            }
        }
    }
    __syncthreads();
    if (abort_flag) {
        if (tid == 0) dd_report_timeout(status);
        return;
    }
    for (int b = 0; b < nb; b++) {
        for (int pi = tid; pi < npix; pi += kThreads) {
            const int r = axis ? line : H - 1 - pi, c = axis ? pi : line;
            const size_t o = ((size_t)(b0 + b) * H + r) * W + c;
            const float val = accs[b * npix + pi];
            if (!add) out[o] = base ? fmaf(scale, val, base[o]) : val;
            else out[o] = base ? fmaf(scale, val, out[o]) : out[o] + val;
        }
    }
}

// Adjoint map of fan beams (plan time): one CTA per (tile, view) fills the
// tile's block.  For each of the tile's walked lines and boundary indices
// b = e - 1 (e from map_first()): the detector bin k and offset u - d_k of the
// clamped boundary value u, exactly as the pixel-gather adjoint needs them
// (k = -1 where the walk does not reach b; boundary i0 - 1 is the walk
// start); then the lines' DD-BP scales.
template <int GEOM>
__global__ void __launch_bounds__(128)
k_amap(dd_geom2d g, int nl, const DdView2 *__restrict__ views, const float *__restrict__ angles,
       const float *__restrict__ dp, const DdLine *__restrict__ lines, unsigned char *__restrict__ amap) {
    const int t = blockIdx.x, v = blockIdx.y;
    const int c0 = (t % tiles_x(&g)) * kTile, r0 = (t / tiles_x(&g)) * kTile;
    const int ms = map_stride(&g), D = g.num_det;
    const DdView2 vw = views[v];
    const int nline = vw.xb ? g.height : g.width;
    const int l0 = vw.xb ? r0 : c0, elo = map_first(&g, vw.xb, c0, r0);
    int2 *ent = reinterpret_cast<int2 *>(amap + ((size_t)v * tiles_n(&g) + t) * kMapBlkBytes);
    float *alpha = reinterpret_cast<float *>(ent + kTile * kMapE);
    const float *dpv = dp + (size_t)v * (D + 1);
    const float ang = angles[v];
    for (int i = threadIdx.x; i < kTile * kMapE; i += 128) {
        const int li = i / kMapE, e = elo + (i - li * kMapE), line = l0 + li;
        int2 val = make_int2(-1, 0);
        if (line < nline && e < ms) {
            const DdLine &L = lines[(size_t)v * nl + line];
            const int b = e - 1, i0 = L.h.i0, nend = L.h.nend;
            if (L.h.npiece > 0 && b >= i0 - 1 && b < nend) {
                const float bound0 = L.h.bound0;
                const float u =
                    (b == i0 - 1) ? bound0 : dd_boundary(&L, b, L.p[0].Q + (float)(b - L.p[0].gb) * L.p[0].dl);
                const float uu = fminf(fmaxf(u, bound0), dpv[D]);
                float dk;
                const int k = fan_bin(GEOM, g, vw, ang, dpv, uu, L.h.idet0, &dk);
                val = make_int2(k, __float_as_int(uu - dk));
            }
        }
        ent[i] = val;
    }
    if (threadIdx.x < kTile) {
        const int line = l0 + threadIdx.x;
        alpha[threadIdx.x] = line < nline ? lines[(size_t)v * nl + line].h.alpha : 0.0f;
    }
}

// Detector-table slice staged per (view, 32x32 tile) by the fan-beam adjoint
// (plan time): the tile's bin range (tile_bin_range) rounded to an even first
// bin and an even count (16-byte bulk copies), or count 0 when wider than the
// staging buffer.  One thread per (view, tile).
template <int GEOM>
__global__ void __launch_bounds__(128)
k_trange(dd_geom2d g, int V, const DdView2 *__restrict__ views, const float *__restrict__ angles,
         int2 *__restrict__ trange) {
    const int nt = tiles_n(&g);
    const int i = blockIdx.x * 128 + threadIdx.x;
    if (i >= V * nt) return;
    const int v = i / nt, t = i - v * nt;
    const int c0 = (t % tiles_x(&g)) * kTile, r0 = (t / tiles_x(&g)) * kTile;
    int kmin, kmax;
    tile_bin_range(GEOM, g, views[v], angles[v], c0, r0, &kmin, &kmax);
    const int rsd = rs_entries(g.num_det);
    const int kb = kmin & ~1;
    int kn = (kmax - kb + 2) & ~1;
    if (kb + kn > rsd) kn = rsd - kb;
    if (kn > kStage || kn <= 0) kn = 0;
    trange[i] = make_int2(kb, kn | (views[v].xb ? 1 << 16 : 0));   // the view's axis in bit 16
}

// Single-geometry adjoint launch: grid (tiles x * image groups, tiles y).
// Fan beams: 4 CTAs per SM (64 registers), as the persistent adjoint.
template <int GEOM, int OPK>
__global__ void __launch_bounds__(kThreads, GEOM == DD_GEOM_PARA ? 1 : 4)
k_adj(dd_geom2d g, int B, int V, int nl, const float *__restrict__ angles,
      const DdView2 *__restrict__ views, const float *__restrict__ dp,
      const DdLine *__restrict__ lines, const DdLine *__restrict__ dlines, const unsigned char *__restrict__ amap,
      const int2 *__restrict__ trange, const float2 *__restrict__ dtab,
      float *__restrict__ out,
      const float *__restrict__ base, float scale, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const AdjSmem SL = adj_smem(GEOM);
    init_bars(reinterpret_cast<uint64_t *>(smem + SL.bar), GEOM == DD_GEOM_PARA ? 2 : kAdjBufs);
    DdPhases ph;
    AdjItem it;
    // the image groups of a tile are adjacent in launch order: they run at the
    // same time, walk the views in step and read each view's map block of the
    // tile once from DRAM between them (the others hit L2)
    const int ngroups = (B + kBI - 1) / kBI;
    it.c0 = (blockIdx.x / ngroups) * kTile;
    it.r0 = blockIdx.y * kTile;
    it.b0 = (blockIdx.x % ngroups) * kBI;
    it.nb = min(kBI, B - it.b0);
    it.V = V;
    it.nl = nl;
    it.angles = angles;
    it.views = views;
    it.dp = dp;
    it.lines = lines;
    it.dlines = dlines;
    it.amap = amap;
    it.trange = trange;
    it.dtab = dtab;
    it.out = out;
    it.base = base;
    it.scale = scale;
    bool ok;
    if constexpr (GEOM == DD_GEOM_PARA) ok = adj_tile<GEOM, OPK>(g, it, smem, ph);
    else ok = adj_tile_map<GEOM, OPK>(g, it, smem, ph);
    if (!ok && threadIdx.x == 0) dd_report_timeout(status);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
int geom_of(int scan) {
    return scan == DD_SCAN_PARA ? DD_GEOM_PARA : (scan == DD_SCAN_FLAT ? DD_GEOM_FLAT : DD_GEOM_ARC);
}

int validate(int scan, int op, const dd_geom2d *g, int B, int V) {
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

int launch_status() {
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

ProfRec *prof_begin(int kind, cudaStream_t st) {
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
void prof_end(ProfRec *r, cudaStream_t st) {
    if (r) cudaEventRecord(r->b, st);
}

void count_launches(int n) { g_launches += (unsigned long long)n; }

int plan(int scan, const dd_geom2d *g, const float *angles, int V, void *planp, size_t bytes,
         cudaStream_t st, bool with_map) {
    const PlanLayout P = plan_layout(scan, g, V, with_map);
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
    if (geom == DD_GEOM_PARA) {
        k_axis_views<<<1, 32, 0, st>>>(V, views, (int *)(base + P.axisv));
        g_launches++;
    }
    dim3 gl((P.nl + 63) / 64, V);
    k_lines<<<gl, 64, 0, st>>>(geom, *g, angles, V, P.nl, views, dp, lines, dlines);
    int n = 2;
    if (geom != DD_GEOM_PARA && with_map) {
        const dim3 gm((unsigned)tiles_n(g), (unsigned)V);
        const float *ang = (const float *)(base + P.ang);
        unsigned char *amap = (unsigned char *)(base + P.amap);
        int2 *trange = (int2 *)(base + P.trange);
        const int nt = (V * tiles_n(g) + 127) / 128;
        if (geom == DD_GEOM_FLAT) {
            k_amap<DD_GEOM_FLAT><<<gm, 128, 0, st>>>(*g, P.nl, views, ang, dp, lines, amap);
            k_trange<DD_GEOM_FLAT><<<nt, 128, 0, st>>>(*g, V, views, ang, trange);
        } else {
            k_amap<DD_GEOM_ARC><<<gm, 128, 0, st>>>(*g, P.nl, views, ang, dp, lines, amap);
            k_trange<DD_GEOM_ARC><<<nt, 128, 0, st>>>(*g, V, views, ang, trange);
        }
        n += 2;
    }
    prof_end(pr, st);
    g_launches += n;
    return launch_status();
}

// Largest dynamic shared memory a CTA may opt in to on this device.
int max_smem_optin() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || n <= 0)
            n = 227 * 1024;   // no device to ask (host-side checks): the sm_103a figure
    }
    return n;
}

template <int GEOM, int BI, int CL>
static auto fwd_kernel(bool w, int D) {
    constexpr int NW = kFwdWarps;
    auto kern = k_fwd<GEOM, 0, 8, NW, BI, CL>;
    switch (npass_class(D, NW)) {
    case 1: kern = w ? k_fwd<GEOM, 1, 1, NW, BI, CL> : k_fwd<GEOM, 0, 1, NW, BI, CL>; break;
    case 2: kern = w ? k_fwd<GEOM, 1, 2, NW, BI, CL> : k_fwd<GEOM, 0, 2, NW, BI, CL>; break;
    case 3: kern = w ? k_fwd<GEOM, 1, 3, NW, BI, CL> : k_fwd<GEOM, 0, 3, NW, BI, CL>; break;
    case 4: kern = w ? k_fwd<GEOM, 1, 4, NW, BI, CL> : k_fwd<GEOM, 0, 4, NW, BI, CL>; break;
    default: kern = w ? k_fwd<GEOM, 1, 8, NW, BI, CL> : k_fwd<GEOM, 0, 8, NW, BI, CL>; break;
    }
    return kern;
}

// The forward CTA shape a tune asks for (slices per CTA, CTAs per view's
// cluster), with the defaults where it asks for none, and 1 slice where the
// line tables of 4 would not fit in shared memory (lines of more than about
// 3,400 pixels).  One slice per CTA keeps a CTA's tables and accumulators
// small (32 registers, 8 CTAs per SM): single-slice calls ran 5-7 % faster
// than with 2 slices per CTA (512^2, 720 views: 0.740 vs 0.789 ms).
static void fwd_shape(int geom, const dd_geom2d *g, const dd_tune2d *tune, int *bi, int *cl) {
    const int rsmax = rs_entries(g->width > g->height ? g->width : g->height);
    *bi = (tune && (tune->fwd_slices == 1 || tune->fwd_slices == 4)) ? tune->fwd_slices : kFwdImages;
    *cl = (tune && (tune->fwd_cluster == 1 || tune->fwd_cluster == 2)) ? tune->fwd_cluster : kFwdCluster;
    if (*bi == 4 && fwd_smem(geom, g->num_det, rsmax, 4, *cl, kFwdWarps).total > max_smem_optin()) *bi = 1;
}

template <int GEOM>
static int launch_fwd(int op, const dd_geom2d *g, const PlanLayout &P, const char *planb, int B,
                      int V, const float2 *tx, const float2 *ty, float *out, const float *sub,
                      int *status, cudaStream_t st, const dd_tune2d *tune) {
    const int rsmax = rs_entries(g->width > g->height ? g->width : g->height);
    const bool w = (op == DD_OP_BPROJ_TW);
    constexpr int NW = kFwdWarps;
    int bi, cl;
    fwd_shape(GEOM, g, tune, &bi, &cl);
    const FwdSmem S = fwd_smem(GEOM, g->num_det, rsmax, bi, cl, NW);
    if (S.total > max_smem_optin()) return DD_ERR_SIZE_OVERFLOW;
    if ((long long)V * cl > 0x7FFFFFFFLL) return DD_ERR_SIZE_OVERFLOW;
    dim3 grid(V * cl, (B + bi - 1) / bi);
    const DdView2 *views = (const DdView2 *)(planb + P.views);
    const float *dp = (const float *)(planb + P.dp);
    const float *bc = (const float *)(planb + P.bcoef);
    const DdLine *lines = (const DdLine *)(planb + P.lines);
    const DdLine *dlines = GEOM == DD_GEOM_PARA ? (const DdLine *)(planb + P.dlines) : nullptr;
    auto kern = (bi == 4) ? (cl == 2 ? fwd_kernel<GEOM, 4, 2>(w, g->num_det) : fwd_kernel<GEOM, 4, 1>(w, g->num_det))
                          : (cl == 2 ? fwd_kernel<GEOM, 1, 2>(w, g->num_det) : fwd_kernel<GEOM, 1, 1>(w, g->num_det));
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S.total) != cudaSuccess)
        return DD_ERR_LAUNCH;
    ProfRec *pr = prof_begin(DD_KERNEL_FORWARD, st);
    kern<<<grid, NW * 32, S.total, st>>>(*g, op, B, V, P.nl, views, dp, bc, lines, dlines, tx, ty,
                                         out, sub, status);
    prof_end(pr, st);
    g_launches++;
    return launch_status();
}

template <int GEOM>
static int launch_adj(int op, const dd_geom2d *g, const PlanLayout &P, const char *planb,
                      const float *angles, int B, int V, const float2 *dtab, float *out,
                      const float *base, float scale, int *status, cudaStream_t st) {
    const unsigned ngroups = (unsigned)((B + kBI - 1) / kBI);
    dim3 grid((unsigned)((g->width + kTile - 1) / kTile) * ngroups, (g->height + kTile - 1) / kTile);
    const DdView2 *views = (const DdView2 *)(planb + P.views);
    const float *dp = (const float *)(planb + P.dp);
    const DdLine *lines = (const DdLine *)(planb + P.lines);
    const DdLine *dlines = GEOM == DD_GEOM_PARA ? (const DdLine *)(planb + P.dlines) : nullptr;
    const unsigned char *amap = GEOM == DD_GEOM_PARA ? nullptr : (const unsigned char *)(planb + P.amap);
    const int2 *trange = GEOM == DD_GEOM_PARA ? nullptr : (const int2 *)(planb + P.trange);
    const AdjSmem S = adj_smem(GEOM);
    auto kern = (op == DD_OP_PROJ_T) ? k_adj<GEOM, 0> : (op == DD_OP_BPROJ) ? k_adj<GEOM, 1> : k_adj<GEOM, 2>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S.total) != cudaSuccess)
        return DD_ERR_LAUNCH;
    ProfRec *pr = prof_begin(DD_KERNEL_ADJOINT, st);
    kern<<<grid, kThreads, S.total, st>>>(*g, B, V, P.nl, angles, views, dp, lines, dlines, amap, trange,
                                          dtab, out, base, scale, status);
    prof_end(pr, st);
    g_launches++;
    return launch_status();
}

// Parallel-beam adjoint: the rows' launch writes, the columns' launch adds.
static int launch_adj_para(int op, const dd_geom2d *g, const PlanLayout &P, const char *planb, int B, int V,
                           const float2 *dtab, float *out, const float *base, float scale, int *status,
                           cudaStream_t st) {
    const DdLine *lines = (const DdLine *)(planb + P.lines);
    const DdLine *dlines = (const DdLine *)(planb + P.dlines);
    const int *axisv = (const int *)(planb + P.axisv);
    const int W = g->width, H = g->height, D = g->num_det;
    const int smax = std::max(para_smem(D, W).total, para_smem(D, H).total);
    if (smax > max_smem_optin()) return DD_ERR_SIZE_OVERFLOW;
    auto kern = (op == DD_OP_PROJ_T) ? k_adj_para<0> : k_adj_para<1>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax) != cudaSuccess)
        return DD_ERR_LAUNCH;
    ProfRec *pr = prof_begin(DD_KERNEL_ADJOINT, st);
    for (int axis = 1; axis >= 0; axis--) {
        const int npix = axis ? W : H, nline = axis ? H : W;
        const dim3 grid((unsigned)nline, (unsigned)((B + kBI - 1) / kBI));
        kern<<<grid, kThreads, para_smem(D, npix).total, st>>>(*g, B, V, P.nl, axis, axisv, lines, dlines, dtab,
                                                                out, base, scale, axis == 0, status);
    }
    prof_end(pr, st);
    g_launches += 2;
    return launch_status();
}

int launch_image_tables(const dd_geom2d *g, const float *in, int B, float2 *tx, float2 *ty,
                        cudaStream_t st) {
    const int W = g->width, H = g->height;
    const int nw = B * H;
    ProfRec *pr = prof_begin(DD_KERNEL_TABLES, st);
    k_tab_rows<<<(nw * 32 + 255) / 256, 256, 0, st>>>(in, B, H, W, tx);
    k_tab_cols<<<B * ((W + 31) / 32), 32 * kColChunks, 0, st>>>(in, B, H, W, ty);
    prof_end(pr, st);
    g_launches += 2;
    return launch_status();
}

int launch_det_tables(int geom, int op, const dd_geom2d *g, const char *planb, const float *in, int B,
                      int V, float2 *dtab, cudaStream_t st) {
    const PlanLayout P = plan_layout(geom == DD_GEOM_PARA ? DD_SCAN_PARA : DD_SCAN_FLAT, g, V);
    const int mode = (op == DD_OP_PROJ_T) ? 0 : 1;
    const float pcx = g->pix_y / g->det_size, pcy = g->pix_x / g->det_size;
    const int nw = B * V;
    ProfRec *pr = prof_begin(DD_KERNEL_TABLES, st);
    k_dettab<<<(nw * 32 + 255) / 256, 256, 0, st>>>(geom, mode, in, B, V, g->num_det,
                                                     (const DdView2 *)(planb + P.views),
                                                     (const float *)(planb + P.dp),
                                                     (const float *)(planb + P.bcoef), pcx, pcy, dtab);
    prof_end(pr, st);
    g_launches++;
    return launch_status();
}

int apply_planned(int scan, int op, const dd_geom2d *g, const void *planp, const float *in,
                  float *out, int B, int V, void *ws, size_t wsb, cudaStream_t st,
                  const float *sub = nullptr, const float *base = nullptr, float scale = 1.0f,
                  const dd_tune2d *tune = nullptr) {
    const PlanLayout P = plan_layout(scan, g, V);
    const float *angles = (const float *)((const char *)planp + P.ang);
    const ApplyLayout A = apply_layout(op, g, B, V);
    if (!ws || wsb < A.total) return DD_ERR_WORKSPACE;
    if (!in || !out || !planp) return DD_ERR_INVALID_ARG;
    const char *planb = (const char *)planp;
    char *wb = (char *)ws;
    int *status = (int *)(wb + A.status);
    const int geom = geom_of(scan);
    if (op_is_forward(op)) {
        float2 *tx = (float2 *)(wb + A.tabx), *ty = (float2 *)(wb + A.taby);
        const int ts = launch_image_tables(g, in, B, tx, ty, st);
        if (ts != DD_OK) return ts;
        if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
        if (geom == DD_GEOM_PARA) return launch_fwd<DD_GEOM_PARA>(op, g, P, planb, B, V, tx, ty, out, sub, status, st, tune);
        if (geom == DD_GEOM_FLAT) return launch_fwd<DD_GEOM_FLAT>(op, g, P, planb, B, V, tx, ty, out, sub, status, st, tune);
        return launch_fwd<DD_GEOM_ARC>(op, g, P, planb, B, V, tx, ty, out, sub, status, st, tune);
    }
    float2 *dtab = (float2 *)(wb + A.dtab);
    const int ts = launch_det_tables(geom, op, g, planb, in, B, V, dtab, st);
    if (ts != DD_OK) return ts;
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    if (geom == DD_GEOM_PARA) return launch_adj_para(op, g, P, planb, B, V, dtab, out, base, scale, status, st);
    if (geom == DD_GEOM_FLAT) return launch_adj<DD_GEOM_FLAT>(op, g, P, planb, angles, B, V, dtab, out, base, scale, status, st);
    return launch_adj<DD_GEOM_ARC>(op, g, P, planb, angles, B, V, dtab, out, base, scale, status, st);
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
    return plan_layout(scan, g, num_view, !op_is_forward(op)).total + apply_layout(op, g, batch, num_view).total;
}

extern "C" int dd2d_plan(int scan, const dd_geom2d *g, const float *angles, int num_view, void *planp,
                         size_t plan_bytes, dd_stream_t stream) {
    ddtrace::Range tr("dd2d_plan", scan, -1, false);
    const int st = validate(scan, DD_OP_PROJ, g, 1, num_view);
    if (st != DD_OK) return st;
    return plan(scan, g, angles, num_view, planp, plan_bytes, (cudaStream_t)stream);
}

extern "C" int dd2d_apply(int scan, int op, const dd_geom2d *g, const float *in, float *out,
                          const float *angles, int batch, int num_view, void *workspace,
                          size_t workspace_bytes, dd_stream_t stream) {
    ddtrace::Range tr("dd2d_apply", scan, op, false);
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!angles || !in || !out) return DD_ERR_INVALID_ARG;
    // a one-shot forward-type call needs no adjoint map in its plan
    const bool with_map = !op_is_forward(op);
    const size_t pb = plan_layout(scan, g, num_view, with_map).total;
    if (!workspace || workspace_bytes < dd2d_workspace_bytes(scan, op, g, batch, num_view))
        return DD_ERR_WORKSPACE;
    const int s1 = plan(scan, g, angles, num_view, workspace, pb, (cudaStream_t)stream, with_map);
    if (s1 != DD_OK) return s1;
    return apply_planned(scan, op, g, workspace, in, out, batch, num_view, (char *)workspace + pb,
                         workspace_bytes - pb, (cudaStream_t)stream);
}

extern "C" int dd2d_apply_planned(int scan, int op, const dd_geom2d *g, const void *planp,
                                  const float *in, float *out, int batch, int num_view,
                                  void *workspace, size_t workspace_bytes, dd_stream_t stream) {
    ddtrace::Range tr("dd2d_apply_planned", scan, op, false);
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    return apply_planned(scan, op, g, planp, in, out, batch, num_view, workspace, workspace_bytes,
                         (cudaStream_t)stream);
}

extern "C" int dd2d_apply_planned_tuned(int scan, int op, const dd_geom2d *g, const void *planp,
                                        const float *in, float *out, int batch, int num_view,
                                        void *workspace, size_t workspace_bytes, const dd_tune2d *tune,
                                        dd_stream_t stream) {
    ddtrace::Range tr("dd2d_apply_planned", scan, op, false);
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    return apply_planned(scan, op, g, planp, in, out, batch, num_view, workspace, workspace_bytes,
                         (cudaStream_t)stream, nullptr, nullptr, 1.0f, tune);
}

extern "C" int dd2d_fwd_shape(int scan, const dd_geom2d *g, const dd_tune2d *tune, int *slices, int *cluster) {
    if (!g || !slices || !cluster || scan < DD_SCAN_PARA || scan > DD_SCAN_ARC) return DD_ERR_INVALID_ARG;
    fwd_shape(geom_of(scan), g, tune, slices, cluster);
    return DD_OK;
}

extern "C" size_t dd2d_dc_workspace_bytes(int scan, const dd_geom2d *g, int batch, int num_view) {
    if (!g || batch <= 0 || num_view <= 0) return 0;
    const size_t a = apply_layout(DD_OP_PROJ, g, batch, num_view).total;
    const size_t b = apply_layout(DD_OP_PROJ_T, g, batch, num_view).total;
    (void)scan;
    return a > b ? a : b;
}

extern "C" int dd2d_dc_step(int scan, const dd_geom2d *g, const void *planp, float *x, const float *y,
                            float *resid, float eta, int batch, int num_view, void *workspace,
                            size_t workspace_bytes, dd_stream_t stream) {
    ddtrace::Range tr("dd2d_dc_step", scan, -1, false);
    const int st = validate(scan, DD_OP_PROJ, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!planp || !x || !y || !resid) return DD_ERR_INVALID_ARG;
    if (!workspace || workspace_bytes < dd2d_dc_workspace_bytes(scan, g, batch, num_view)) return DD_ERR_WORKSPACE;
    cudaStream_t s = (cudaStream_t)stream;
    const int s1 = apply_planned(scan, DD_OP_PROJ, g, planp, x, resid, batch, num_view, workspace,
                                 workspace_bytes, s, y);
    if (s1 != DD_OK) return s1;
    return apply_planned(scan, DD_OP_PROJ_T, g, planp, resid, x, batch, num_view, workspace, workspace_bytes,
                         s, nullptr, x, -eta);
}

static int read_word(const void *p, int *status) {
    if (cudaMemcpy(status, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return DD_ERR_LAUNCH;
    return DD_OK;
}

extern "C" int dd2d_status(int scan, int op, const dd_geom2d *g, int batch, int num_view, const void *workspace,
                           int *status) {
    if (validate(scan, op, g, batch, num_view) != DD_OK || !workspace || !status) return DD_ERR_INVALID_ARG;
    const size_t pb = plan_layout(scan, g, num_view, !op_is_forward(op)).total;
    return read_word((const char *)workspace + pb + apply_layout(op, g, batch, num_view).status, status);
}

extern "C" int dd2d_planned_status(int op, const dd_geom2d *g, int batch, int num_view, const void *workspace,
                                   int *status) {
    if (!g || batch <= 0 || num_view <= 0 || !workspace || !status) return DD_ERR_INVALID_ARG;
    return read_word((const char *)workspace + apply_layout(op, g, batch, num_view).status, status);
}

// byte offset of the status word of a dd2d_apply call in its workspace (used by
// the no-allocation entry point, whose workspace is the library's own buffer)
size_t dd2d_status_offset(int scan, int op, const dd_geom2d *g, int batch, int num_view) {
    return plan_layout(scan, g, num_view, !op_is_forward(op)).total + apply_layout(op, g, batch, num_view).status;
}

// each translation unit with bounded waits keeps its own sink pointer
int dd2b_set_sink(int *sink);   // dd2d_batch.cu
int dd3_set_sink(int *sink);    // dd3d.cu

extern "C" int dd_set_status_sink(int *sink) {
    int *dev_ptr = nullptr;
    if (sink && cudaHostGetDevicePointer((void **)&dev_ptr, sink, 0) != cudaSuccess) {
        (void)cudaGetLastError();
        return DD_ERR_INVALID_ARG;   // not pinned, device-mapped host memory
    }
    if (dd_set_status_sink_tu(dev_ptr) || dd2b_set_sink(dev_ptr) || dd3_set_sink(dev_ptr)) return DD_ERR_LAUNCH;
    return DD_OK;
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

extern "C" const char *dd_version(void) { return "pridediff_dd 0.2 sm_103a"; }

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
