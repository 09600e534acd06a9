// 3-D DD projector (cone-flat, cone-arc, spiral): plan kernels, the
// forward-type kernel (detector gathers) and the adjoint-type kernel (voxel
// gathers), and the C ABI of include/pridediff_dd.h for the 18 3-D
// radontorch operators (RadonTorch.cpp:1395-1414).
//
// Forward-type operators (Proj, BackProjTrans, BackProjTransWeighted): one
// thread per (view, column, 8 detector rows, 2 volumes) loops over the walked
// image lines; for each line it enumerates the overlap segments of its
// column with the drifted pixel boundaries (dd3_colwalk_*), then walks the
// slices each of its rows meets and gathers voxels.  Volumes are read from a
// transposed copy for views that walk image columns, so that the pixels of a
// walked line are contiguous in both branches.
//
// Adjoint-type operators (ProjTrans, BackProj, BackProjWeighted): one thread
// per (x, y) voxel column, 8 slices and 2 volumes loops over the views; for
// each view it enumerates the segments of its pixel with the detector columns
// (dd3_pixwalk_*) and gathers the rows that meet each slice from a sinogram
// pre-multiplied by the per-bin scale.  A per-CTA test skips views whose
// detector cannot see the CTA's slab (most views of a spiral scan).
//
// Both directions use the same segment widths and z-walk widths, so they are
// exact transposes of each other; no atomics, deterministic results.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pridediff_dd.h"
#include "dd_geom3d.cuh"
#include "dd_tma.cuh"
#include "dd_trace.h"

namespace dd2 {   // launch accounting and profiling (dd2d.cu)
struct ProfRec;
ProfRec *prof_begin(int kind, cudaStream_t st);
void prof_end(ProfRec *r, cudaStream_t st);
void count_launches(int n);
}   // namespace dd2

namespace dd3 {

constexpr int kThreads = 256;
constexpr int kNB = 2;     // volumes per thread
constexpr int kTile = 16;  // adjoint: 16 x 16 voxel columns per CTA
constexpr int kZS = 8;     // adjoint: slices per thread

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// Layouts
// ---------------------------------------------------------------------------
// Per-view tables are padded to 16-byte rows so that one view's row can be
// moved by a single bulk copy: dp (C+1 column boundaries), mag (C column
// magnifications), rowz (R x {row0z, row1z}).
struct PlanLayout {
    size_t views, dp, mag, rowz, linez, lines, slabv, total;
    int nl, nch, sdp, smag, srz, nslab;
};

__host__ __device__ inline int pad4(int n) { return (n + 3) & ~3; }

inline PlanLayout plan_layout(const dd_geom3d *g, int V) {
    PlanLayout L;
    const int C = g->num_col, R = g->num_row;
    L.nl = g->height > g->width ? g->height : g->width;
    L.nch = (C + DD3_CHUNK - 1) / DD3_CHUNK;
    L.sdp = pad4(C + 1);
    L.smag = pad4(C);
    L.srz = pad4(2 * R);
    size_t o = 0;
    L.views = o; o = align_up(o + sizeof(DdView3) * (size_t)V, 256);
    L.dp = o; o = align_up(o + sizeof(float) * (size_t)V * L.sdp, 256);
    L.mag = o; o = align_up(o + sizeof(float) * (size_t)V * L.smag, 256);
    L.rowz = o; o = align_up(o + sizeof(float) * (size_t)V * L.srz, 256);
    L.linez = o; o = align_up(o + sizeof(float4) * (size_t)V * L.nl, 256);
    L.lines = o; o = align_up(o + sizeof(DdLine) * (size_t)V * L.nl * L.nch, 256);
    L.nslab = (g->depth + kZS - 1) / kZS;   // the adjoint's slabs of kZS slices
    L.slabv = o; o = align_up(o + sizeof(int2) * (size_t)L.nslab, 256);
    L.total = o;
    return L;
}

struct ApplyLayout {
    size_t volT, ss, status, total;
};

inline bool op_is_forward(int op) { return op == DD_OP_PROJ || op == DD_OP_BPROJ_T || op == DD_OP_BPROJ_TW; }
inline int op_family(int op) {
    return (op == DD_OP_PROJ || op == DD_OP_PROJ_T) ? 0 : (op == DD_OP_BPROJ_W || op == DD_OP_BPROJ_TW) ? 2 : 1;
}

// fwd / adj select which scratch areas are needed (both for the DC step)
inline ApplyLayout apply_layout(bool fwd, bool adj, const dd_geom3d *g, int B, int V) {
    ApplyLayout L;
    size_t o = 0;
    L.volT = L.ss = 0;
    if (fwd) { L.volT = o; o = align_up(o + sizeof(float) * (size_t)B * g->depth * g->width * g->height, 256); }
    if (adj) { L.ss = o; o = align_up(o + sizeof(float) * (size_t)B * V * g->num_row * g->num_col, 256); }
    L.status = o; o = align_up(o + 256, 256);
    L.total = o;
    return L;
}

// ---------------------------------------------------------------------------
// Plan kernels
// ---------------------------------------------------------------------------
// One CTA per view: scalars, column boundaries, column magnifications, row
// table, and the ranges used by the adjoint's candidate searches.
template <int GEOM>
__global__ void __launch_bounds__(kThreads) k_views3(dd_geom3d g, const float *__restrict__ angles,
                                                     const float *__restrict__ sp, int V, char *plan,
                                                     PlanLayout P) {
    const int v = blockIdx.x, tid = threadIdx.x;
    const int C = g.num_col, R = g.num_row;
    __shared__ DdView3 sw;
    __shared__ float red[2][kThreads / 32];
    if (tid == 0) {
        float sp4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (GEOM == DD_GEOM3_SPIRAL)
            for (int i = 0; i < 4; i++) sp4[i] = sp[(size_t)i * V + v];
        dd3_view_scalars(GEOM, &g, angles[v], sp4, &sw);
    }
    __syncthreads();
    const DdView3 w = sw;
    float *dp = reinterpret_cast<float *>(plan + P.dp) + (size_t)v * P.sdp;
    float *mag = reinterpret_cast<float *>(plan + P.mag) + (size_t)v * P.smag;
    float *rz = reinterpret_cast<float *>(plan + P.rowz) + (size_t)v * P.srz;
    for (int k = tid; k <= C; k += kThreads) dp[k] = dd3_col_boundary(GEOM, &g, &w, k);
    float mn = 3.0e38f, mx = -3.0e38f;
    for (int k = tid; k < C; k += kThreads) {
        const float m = dd3_col_mag(GEOM, &g, &w, k);
        mag[k] = m;
        mn = fminf(mn, m);
        mx = fmaxf(mx, m);
    }
    for (int r = tid; r < R; r += kThreads) dd3_row_z(GEOM, &g, &w, r, &rz[2 * r], &rz[2 * r + 1]);
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = mn;
        red[1][tid >> 5] = mx;
    }
    __syncthreads();
    if (tid == 0) {
        DdView3 out = w;
        out.magmin = red[0][0];
        out.magmax = red[1][0];
        for (int i = 1; i < kThreads / 32; i++) {
            out.magmin = fminf(out.magmin, red[0][i]);
            out.magmax = fmaxf(out.magmax, red[1][i]);
        }
        float a0, a1, b0, b1;
        dd3_row_z(GEOM, &g, &w, 0, &a0, &a1);
        dd3_row_z(GEOM, &g, &w, R - 1, &b0, &b1);
        out.rzA = a0;
        out.rzB = (R > 1) ? (b0 - a0) / (float)(R - 1) : a1 - a0;
        reinterpret_cast<DdView3 *>(plan + P.views)[v] = out;
    }
}

// One thread per (view, line, walk block): walk start and drift pieces.
template <int GEOM>
__global__ void __launch_bounds__(128) k_lines3(dd_geom3d g, char *plan, PlanLayout P) {
    const int v = blockIdx.y;
    const int idx = blockIdx.x * 128 + threadIdx.x;
    const int line = idx / P.nch, cc = idx - line * P.nch;
    const DdView3 *views = reinterpret_cast<const DdView3 *>(plan + P.views);
    const int xb = views[v].xb;
    const int nline = xb ? g.height : g.width;
    if (line >= nline) return;
    const DdView3 w = views[v];
    const float *dp = reinterpret_cast<const float *>(plan + P.dp) + (size_t)v * P.sdp;
    DdLine *L = reinterpret_cast<DdLine *>(plan + P.lines) + ((size_t)v * P.nl + line) * P.nch + cc;
    float lz[4];
    dd3_line_setup(GEOM, &g, &w, dp, line, cc, lz, L);
    if (cc == 0)
        reinterpret_cast<float4 *>(plan + P.linez)[(size_t)v * P.nl + line] = make_float4(lz[0], lz[1], lz[2], lz[3]);
}

// volT[b][s][x][H-1-y] = vol[b][s][y][x]: walked lines of y-branch views
// become contiguous rows.
__global__ void __launch_bounds__(256) k_transpose3(const float *__restrict__ in, float *__restrict__ out, int W,
                                                    int H, int nplanes) {
    __shared__ float t[32][33];
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int pl = blockIdx.z; pl < nplanes; pl += gridDim.z) {
        const size_t plane = (size_t)pl * W * H;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int y = y0 + ty + 8 * i, x = x0 + tx;
            if (y < H && x < W) t[ty + 8 * i][tx] = in[plane + (size_t)y * W + x];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int x = x0 + ty + 8 * i, y = y0 + tx;
            if (x < W && y < H) out[plane + (size_t)x * H + (H - 1 - y)] = t[tx][ty + 8 * i];
        }
        __syncthreads();
    }
}

// ss[b][v][r][k] = in[b][v][r][k'] * scale(v, r, k) with k the sorted column:
// the adjoint gathers pre-scaled bins (ConeFlatDisCUDA3d.cu:400-404).
template <int GEOM, int FAMILY>
__global__ void __launch_bounds__(128) k_sino3(dd_geom3d g, const char *__restrict__ plan, PlanLayout P,
                                               const float *__restrict__ in, float *__restrict__ ss, int B, int V) {
    const int C = g.num_col, R = g.num_row;
    const int k = blockIdx.x * 128 + threadIdx.x, r = blockIdx.y, v = blockIdx.z;
    if (k >= C) return;
    const DdView3 &w = reinterpret_cast<const DdView3 *>(plan + P.views)[v];
    float scale = w.bp_scale;
    if (FAMILY == 0) {
        const float *dp = reinterpret_cast<const float *>(plan + P.dp) + (size_t)v * P.sdp;
        const float *rz = reinterpret_cast<const float *>(plan + P.rowz) + (size_t)v * P.srz;
        const float mag = reinterpret_cast<const float *>(plan + P.mag)[(size_t)v * P.smag + k];
        float rp0, rp1;
        dd3_rp(GEOM, &w, mag, rz[2 * r], rz[2 * r + 1], &rp0, &rp1);
        scale = dd3_proj_scale(&g, &w, dp[k], dp[k + 1], rp0, rp1);
    }
    const int ko = w.flip ? C - 1 - k : k;
    const size_t per = (size_t)V * R * C;
    const size_t row = ((size_t)v * R + r) * C;
    for (int b = 0; b < B; b++) ss[b * per + row + k] = FMUL(in[b * per + row + ko], scale);
}

// ---------------------------------------------------------------------------
// Forward-type kernel: detector gathers
// ---------------------------------------------------------------------------
constexpr int kFC = 32;    // detector columns per CTA (the lanes of a warp)
// Forward CTA: 8 consumer warps x 4 consecutive detector rows per thread =
// 32 rows, plus a producer warp that turns each line's record into column
// segments one line ahead; 3 CTAs per SM at 72 registers.
constexpr int kFR = 4;
constexpr int kFwdWarps3 = 8;                          // consumer warps
constexpr int kFwdThreads3 = (kFwdWarps3 + 1) * 32;   // + the producer warp
constexpr int kSeg = 8;    // column segments of one line held in shared memory

struct Fwd3Args {
    dd_geom3d g;
    const char *plan;
    PlanLayout P;
    const float *vol;    // (B, Dep, H, W)
    const float *volT;   // (B, Dep, W, H), pixel order reversed along y
    float *out;          // (B, V, R, C)
    const float *sub;    // optional: out = A x - sub
    int *status;
    int B, V, nrb;
};

// grid: (view, group of 32 columns inside one walk block, row block x volume
// group).  Lane = column, consumer warp w = rows r0 + 4w .. r0 + 4w + 3, kNB
// volumes.  The overlap segments of a line (pixel, width x operator factor)
// depend on the column only, so they are computed once per line and column
// -- by the producer warp, one line ahead, while the consumer warps walk the
// current line -- into shared memory, and reused by all 32 rows.  Line
// records arrive by bulk copies (TMA) two lines ahead.
template <int GEOM, int FAMILY>
__global__ void __launch_bounds__(kFwdThreads3, 3) k_fwd3(const Fwd3Args a) {
    const dd_geom3d &g = a.g;
    const int W = g.width, H = g.height, Dp = g.depth, C = g.num_col, R = g.num_row;
    const int v = blockIdx.x, cg = blockIdx.y;
    const int rb = blockIdx.z % a.nrb, bg = blockIdx.z / a.nrb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cc = (cg * kFC) / DD3_CHUNK, c0 = cc * DD3_CHUNK;
    const int k = cg * kFC + lane, kk = k - c0;
    const bool active = k < C;
    const bool prod = warp == kFwdWarps3;   // the producer warp owns no rows
    const int r0 = rb * (kFR * kFwdWarps3) + warp * kFR, b0 = bg * kNB;
    const int nb = min(kNB, a.B - b0);
    const PlanLayout &P = a.P;

    __shared__ __align__(128) DdLine srec[2];
    __shared__ __align__(16) float4 slzr[2];        // z quantities arriving with each record
    __shared__ __align__(16) float4 slz[2];         // z quantities of the segment buffers
    __shared__ int segj[2][kSeg][kFC];
    __shared__ float segc[2][kSeg][kFC];
    __shared__ int segn[2][kFC];
    __shared__ float sdp[kFC + 1];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int abort_flag, nissue[2], nwait[2];   // copies issued / waited per record buffer

    const DdView3 w = reinterpret_cast<const DdView3 *>(a.plan + P.views)[v];
    const float *__restrict__ dpv = reinterpret_cast<const float *>(a.plan + P.dp) + (size_t)v * P.sdp;
    const float *__restrict__ rz = reinterpret_cast<const float *>(a.plan + P.rowz) + (size_t)v * P.srz;
    const float4 *__restrict__ linez = reinterpret_cast<const float4 *>(a.plan + P.linez) + (size_t)v * P.nl;
    const DdLine *__restrict__ lines = reinterpret_cast<const DdLine *>(a.plan + P.lines) + (size_t)v * P.nl * P.nch + cc;
    if (tid <= kFC) sdp[tid] = dpv[min(cg * kFC + tid, C)];
    if (tid == 0) {
        abort_flag = 0;
        nissue[0] = nissue[1] = nwait[0] = nwait[1] = 0;
        dd_mbar_init(&bar[0], 1);
        dd_mbar_init(&bar[1], 1);
        dd_fence_mbar_init();
    }
    __syncthreads();

    const int xb = w.xb;
    const int nline = xb ? H : W, npix = xb ? W : H;
    auto issue = [&](int line, int buf) {
        nissue[buf]++;
        dd_mbar_expect_tx(&bar[buf], (uint32_t)(sizeof(DdLine) + sizeof(float4)));
        dd_bulk_g2s(&srec[buf], lines + (size_t)line * P.nch, (uint32_t)sizeof(DdLine), &bar[buf]);
        dd_bulk_g2s(&slzr[buf], linez + line, (uint32_t)sizeof(float4), &bar[buf]);
    };
    // segments of line m (record buffer m & 1) into segment buffer sb; one warp
    auto produce = [&](int m, int sb) -> bool {
        const int rbuf = m & 1;
        const uint32_t parity = (uint32_t)nwait[rbuf] & 1u;
        if (!dd_mbar_wait(&bar[rbuf], parity)) return false;
        const DdLine *L = &srec[rbuf];
        const float4 lz = slzr[rbuf];
        if (lane == 0) slz[sb] = lz;
        int n = 0;
        DdColWalk cw;
        if (active && dd3_colwalk_init(L, sdp, lane, kk, &cw)) {
            const float lpos = (FAMILY == 2) ? dd3_line_pos(&g, &w, m) : 0.0f;
            int j;
            float wd;
            while (dd3_colwalk_next(L, &cw, &j, &wd)) {
                if (n == kSeg) {   // more than kSeg segments: consumers walk the record themselves
                    n = kSeg + 1;
                    break;
                }
                segj[sb][n][lane] = j;
                segc[sb][n][lane] = dd3_coef(GEOM, FAMILY, &g, &w, lpos, j, wd, lz.w);
                n++;
            }
        }
        segn[sb][lane] = n;
        __syncwarp();
        if (lane == 0) nwait[rbuf]++;
        return true;
    };

    float rp0[kFR], rp1[kFR];
    {
        const float mag = active ? reinterpret_cast<const float *>(a.plan + P.mag)[(size_t)v * P.smag + k] : 1.0f;
#pragma unroll
        for (int q = 0; q < kFR; q++) {
            const int r = r0 + q;
            if (active && !prod && r < R) {
                dd3_rp(GEOM, &w, mag, rz[2 * r], rz[2 * r + 1], &rp0[q], &rp1[q]);
            } else {
                rp0[q] = 3.0e38f;    // empty row: the z walk never starts
                rp1[q] = -3.0e38f;
            }
        }
    }
    float acc[kFR][kNB];
#pragma unroll
    for (int q = 0; q < kFR; q++)
#pragma unroll
        for (int b = 0; b < kNB; b++) acc[q][b] = 0.0f;

    const float *__restrict__ src = xb ? a.vol : a.volT;
    const size_t plane = (size_t)nline * npix;
    const size_t vstride = (size_t)Dp * plane;
    src += (size_t)b0 * vstride;

    // prologue: records 0 and 1 in flight, segments of line 0 computed
    if (tid == 0) {
        issue(0, 0);
        if (nline > 1) issue(1, 1);
    }
    __syncthreads();
    if (prod && !produce(0, 0)) abort_flag = 1;
    __syncthreads();
    if (tid == 0 && !abort_flag && nline > 2) issue(2, 0);
    for (int line = 0; line < nline && !abort_flag; line++) {
        const int sb = line & 1;
        if (line + 1 < nline && prod && !produce(line + 1, sb ^ 1)) abort_flag = 1;
        // consume line `line`
        const int n = segn[sb][lane];
        if (active && !prod && n > 0) {
            const float4 lz = slz[sb];
            const float *__restrict__ lsrc = src + (size_t)line * npix;
            if (n <= kSeg) {
#pragma unroll
                for (int q = 0; q < kFR; q++) {
                    const float bz0 = fmaxf(lz.x, rp0[q]), bz1 = fminf(lz.y, rp1[q]);
                    if (!(bz0 < bz1)) continue;
                    int s = dd3_slice_first(bz0, lz.x, lz.z);
                    float zhi = dd3_zb(lz.x, lz.z, s);
                    for (; s < Dp; s++) {
                        const float zlo = zhi;
                        if (!(zlo < bz1)) break;
                        zhi = dd3_zb(lz.x, lz.z, s + 1);
                        const float zw = dd3_cell(bz0, bz1, zlo, zhi);
                        if (!(zw > 0.0f)) continue;
                        const float *__restrict__ ps = lsrc + (size_t)s * plane;
                        for (int t = 0; t < n; t++) {
                            const float wq = FMUL(zw, segc[sb][t][lane]);
                            const int j = segj[sb][t][lane];
#pragma unroll
                            for (int b = 0; b < kNB; b++)
                                if (b < nb) acc[q][b] = fmaf(wq, __ldg(ps + (size_t)b * vstride + j), acc[q][b]);
                        }
                    }
                }
            } else {
                // wide column: walk the record in global memory
                const DdLine *Lg = lines + (size_t)line * P.nch;
                const float lpos = (FAMILY == 2) ? dd3_line_pos(&g, &w, line) : 0.0f;
                DdColWalk cw;
                if (dd3_colwalk_init(Lg, sdp, lane, kk, &cw)) {
                    int j;
                    float wd;
                    while (dd3_colwalk_next(Lg, &cw, &j, &wd)) {
                        const float cf = dd3_coef(GEOM, FAMILY, &g, &w, lpos, j, wd, lz.w);
#pragma unroll
                        for (int q = 0; q < kFR; q++) {
                            const float bz0 = fmaxf(lz.x, rp0[q]), bz1 = fminf(lz.y, rp1[q]);
                            if (!(bz0 < bz1)) continue;
                            for (int s = dd3_slice_first(bz0, lz.x, lz.z); s < Dp; s++) {
                                const float zlo = dd3_zb(lz.x, lz.z, s);
                                if (!(zlo < bz1)) break;
                                const float zw = dd3_cell(bz0, bz1, zlo, dd3_zb(lz.x, lz.z, s + 1));
                                if (!(zw > 0.0f)) continue;
                                const float wq = FMUL(zw, cf);
                                const float *__restrict__ ps = lsrc + (size_t)s * plane + j;
#pragma unroll
                                for (int b = 0; b < kNB; b++)
                                    if (b < nb) acc[q][b] = fmaf(wq, __ldg(ps + (size_t)b * vstride), acc[q][b]);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        // the record of line + 1 has been turned into segments: its buffer takes line + 3
        if (tid == 0 && !abort_flag && line + 3 < nline) issue(line + 3, (line + 1) & 1);
    }
    __syncthreads();
    if (abort_flag) {
        // let copies still in flight land before the CTA exits
        if (tid == 0) {
            for (int b = 0; b < 2; b++)
                if (nissue[b] > nwait[b]) dd_mbar_drain(&bar[b], (uint32_t)nwait[b] & 1u);
            dd_report_timeout(a.status);
        }
        return;
    }
    if (!active || prod) return;
    const int ko = w.flip ? C - 1 - k : k;
#pragma unroll
    for (int q = 0; q < kFR; q++) {
        const int r = r0 + q;
        if (r >= R) continue;
        const float scale = (FAMILY == 0) ? dd3_proj_scale(&g, &w, sdp[lane], sdp[lane + 1], rp0[q], rp1[q]) : w.bp_scale;
#pragma unroll
        for (int b = 0; b < kNB; b++) {
            if (b < nb) {
                const size_t o = (((size_t)(b0 + b) * a.V + v) * R + r) * C + ko;
                float val = FMUL(acc[q][b], scale);
                if (a.sub) val = FSUB(val, a.sub[o]);
                a.out[o] = val;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint-type kernel: voxel gathers
// ---------------------------------------------------------------------------
struct Adj3Args {
    dd_geom3d g;
    const char *plan;
    PlanLayout P;
    const float *ss;     // pre-scaled sinogram (B, V, R, C), sorted columns
    float *out;          // (B, Dep, H, W)
    const float *base;   // optional: out = base + scale * value (may alias out)
    float scale;
    int *status;
    int B, V, ntx;
};

// Shared memory of the adjoint kernel: two buffers of one view's data (the
// records of the tile's 16 lines in every walk block, the column boundary,
// column magnification and row tables, the lines' z quantities and the view
// record), each moved by bulk copies; all sizes are multiples of 16 bytes.
struct Adj3Smem {
    int rec, dp, mag, rz, lz, vw, bar, total;
    uint32_t rec_b, dp_b, mag_b, rz_b, lz_b;
};

__host__ __device__ inline Adj3Smem adj3_smem(const PlanLayout &P) {
    Adj3Smem s;
    s.rec_b = (uint32_t)(kTile * P.nch * sizeof(DdLine));
    s.dp_b = (uint32_t)(P.sdp * sizeof(float));
    s.mag_b = (uint32_t)(P.smag * sizeof(float));
    s.rz_b = (uint32_t)(P.srz * sizeof(float));
    s.lz_b = (uint32_t)(kTile * sizeof(float4));
    int o = 0;
    s.rec = o; o += 2 * (int)s.rec_b;
    s.dp = o; o += 2 * (int)s.dp_b;
    s.mag = o; o += 2 * (int)s.mag_b;
    s.rz = o; o += 2 * (int)s.rz_b;
    s.lz = o; o += 2 * (int)s.lz_b;
    s.vw = o; o += 2 * (int)sizeof(DdView3);
    s.bar = o; o += 2 * (int)sizeof(uint64_t);
    s.total = (o + 127) & ~127;
    return s;
}

// Can view w see the slab of slices [s0, s0 + kZS) on the walked lines
// l0..l1 (with one slice of margin)?
__device__ __forceinline__ bool slab_visible(const dd_geom3d &g, const DdView3 &w, int l0, int l1, int s0,
                                             float zr0, float zr1) {
    const float m0 = dd3_line_mag(&w, dd3_line_pos(&g, &w, l0));
    const float m1 = dd3_line_mag(&w, dd3_line_pos(&g, &w, l1));
    const float zsA = w.z0 + (float)(s0 - 1) * g.pix_z, zsB = w.z0 + (float)(s0 + kZS + 1) * g.pix_z;
    return dd3_slab_lit(&w, fminf(m0, m1), fmaxf(m0, m1), zsA, zsB, zr0, zr1);
}

// Plan time: for each slab of kZS slices, the views [first, last] whose
// detector can see it anywhere in the image -- slab_visible over the whole
// image's lines, a superset of what it admits for any tile's lines (wider
// magnification bounds only widen the lit band) -- stored as {first,
// last + 1}, {0, 0} if none.  The adjoint loops over these views only: on a
// spiral a slab is lit during one pass of the helix.
__global__ void __launch_bounds__(256) k_slab_views3(dd_geom3d g, char *plan, PlanLayout P, int V) {
    const int slab = blockIdx.x, R = g.num_row;
    const DdView3 *views = reinterpret_cast<const DdView3 *>(plan + P.views);
    const float *rzt = reinterpret_cast<const float *>(plan + P.rowz);
    __shared__ int lo, hi;
    if (threadIdx.x == 0) {
        lo = V;
        hi = -1;
    }
    __syncthreads();
    int mylo = V, myhi = -1;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const DdView3 w = views[v];
        const int nline = w.xb ? g.height : g.width;
        const float *rzv = rzt + (size_t)v * P.srz;
        if (slab_visible(g, w, 0, nline - 1, slab * kZS, rzv[0], rzv[2 * R - 1])) {
            mylo = min(mylo, v);
            myhi = max(myhi, v);
        }
    }
    atomicMin(&lo, mylo);
    atomicMax(&hi, myhi);
    __syncthreads();
    if (threadIdx.x == 0)
        reinterpret_cast<int2 *>(plan + P.slabv)[slab] = hi >= lo ? make_int2(lo, hi + 1) : make_int2(0, 0);
}

// grid: (voxel-column tile, slab of kZS slices, volume group); thread = one
// (x, y) voxel column of a 16 x 16 tile.  Views whose detector cannot see the
// slab are skipped when their copy would be issued.
template <int GEOM, int FAMILY>
__global__ void __launch_bounds__(kThreads, 3) k_adj3(const Adj3Args a) {
    extern __shared__ __align__(128) unsigned char sm[];
    const dd_geom3d &g = a.g;
    const int W = g.width, H = g.height, Dp = g.depth, C = g.num_col, R = g.num_row;
    const PlanLayout &P = a.P;
    const Adj3Smem S = adj3_smem(P);
    const int tid = threadIdx.x;
    const int tX = blockIdx.x % a.ntx, tY = blockIdx.x / a.ntx;
    const int xlo = tX * kTile, ylo = tY * kTile;
    const int x = xlo + (tid & (kTile - 1)), y = ylo + (tid / kTile);
    const bool active = x < W && y < H;
    const int s0 = blockIdx.y * kZS, b0 = blockIdx.z * kNB;
    const int nb = min(kNB, a.B - b0);
    const DdView3 *__restrict__ views = reinterpret_cast<const DdView3 *>(a.plan + P.views);
    const float *__restrict__ dpt = reinterpret_cast<const float *>(a.plan + P.dp);
    const float *__restrict__ magt = reinterpret_cast<const float *>(a.plan + P.mag);
    const float *__restrict__ rzt = reinterpret_cast<const float *>(a.plan + P.rowz);
    const float4 *__restrict__ linez = reinterpret_cast<const float4 *>(a.plan + P.linez);
    const DdLine *__restrict__ lines = reinterpret_cast<const DdLine *>(a.plan + P.lines);
    const size_t per = (size_t)a.V * R * C;
    const float *__restrict__ ssb = a.ss + (size_t)b0 * per;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + S.bar);
    __shared__ int abort_flag;
    __shared__ int seen[2];   // per buffer: 1 if the view sees the slab (data copied)

    if (tid == 0) {
        abort_flag = 0;
        dd_mbar_init(&bar[0], 1);
        dd_mbar_init(&bar[1], 1);
        dd_fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int v, int buf) {
        const DdView3 wv = views[v];
        const int xbv = wv.xb;
        const int l0 = xbv ? ylo : xlo;
        const int n = min(kTile, (xbv ? H : W) - l0);
        const float *rzv = rzt + (size_t)v * P.srz;
        const bool lit = slab_visible(g, wv, l0, l0 + n - 1, s0, rzv[0], rzv[2 * R - 1]);
        seen[buf] = lit ? 1 : 0;
        if (!lit) {
            dd_mbar_expect_tx(&bar[buf], 0u);   // completes the phase with no data
            return;
        }
        const uint32_t rb = (uint32_t)(n * P.nch * sizeof(DdLine)), lb = (uint32_t)(n * sizeof(float4));
        dd_mbar_expect_tx(&bar[buf], rb + S.dp_b + S.mag_b + S.rz_b + lb + (uint32_t)sizeof(DdView3));
        dd_bulk_g2s(sm + S.rec + buf * S.rec_b, lines + ((size_t)v * P.nl + l0) * P.nch, rb, &bar[buf]);
        dd_bulk_g2s(sm + S.dp + buf * S.dp_b, dpt + (size_t)v * P.sdp, S.dp_b, &bar[buf]);
        dd_bulk_g2s(sm + S.mag + buf * S.mag_b, magt + (size_t)v * P.smag, S.mag_b, &bar[buf]);
        dd_bulk_g2s(sm + S.rz + buf * S.rz_b, rzv, S.rz_b, &bar[buf]);
        dd_bulk_g2s(sm + S.lz + buf * S.lz_b, linez + (size_t)v * P.nl + l0, lb, &bar[buf]);
        dd_bulk_g2s(sm + S.vw + buf * (int)sizeof(DdView3), views + v, (uint32_t)sizeof(DdView3), &bar[buf]);
    };

    float acc[kZS][kNB];
#pragma unroll
    for (int q = 0; q < kZS; q++)
#pragma unroll
        for (int b = 0; b < kNB; b++) acc[q][b] = 0.0f;

    DdPhases ph;
    int inflight = -1;
    // only the views that can see this slab somewhere in the image
    const int2 vr = reinterpret_cast<const int2 *>(a.plan + P.slabv)[blockIdx.y];
    if (tid == 0 && vr.x < vr.y) issue(vr.x, 0);
    for (int v = vr.x; v < vr.y; v++) {
        const int buf = (v - vr.x) & 1;
        if (tid == 0 && v + 1 < vr.y) issue(v + 1, buf ^ 1);
        if (!dd_mbar_wait(&bar[buf], ph.parity(buf))) abort_flag = 1;
        ph.flip(buf);
        __syncthreads();
        if (abort_flag) {
            // view v's copies (the wait gave up on them) and view v + 1's may be in flight
            if (tid == 0) dd_mbar_drain(&bar[buf], ph.parity(buf) ^ 1u);
            inflight = (v + 1 < vr.y) ? (buf ^ 1) : -1;
            break;
        }
        if (active && seen[buf]) {
            const DdView3 &w = *reinterpret_cast<const DdView3 *>(sm + S.vw + buf * (int)sizeof(DdView3));
            const float *dp = reinterpret_cast<const float *>(sm + S.dp + buf * S.dp_b);
            const float *mg = reinterpret_cast<const float *>(sm + S.mag + buf * S.mag_b);
            const float *rz = reinterpret_cast<const float *>(sm + S.rz + buf * S.rz_b);
            const int xb = w.xb;
            const int rl = xb ? (y - ylo) : (x - xlo);
            const int line = (xb ? ylo : xlo) + rl;
            const int j = xb ? x : H - 1 - y;
            const float4 lz = reinterpret_cast<const float4 *>(sm + S.lz + buf * S.lz_b)[rl];
            const DdLine *lrec = reinterpret_cast<const DdLine *>(sm + S.rec + buf * S.rec_b) + rl * P.nch;
            const float lpos = (FAMILY == 2) ? dd3_line_pos(&g, &w, line) : 0.0f;
            float zb[kZS + 1];   // slice boundaries of the slab on this line
#pragma unroll
            for (int q = 0; q <= kZS; q++) zb[q] = dd3_zb(lz.x, lz.z, s0 + q);
            const float *__restrict__ ssv = ssb + (size_t)v * R * C;
            for (int cc = 0; cc < P.nch; cc++) {
                DdPixWalk pw;
                if (!dd3_pixwalk_init(GEOM, &g, &w, lrec + cc, dp, cc, j, &pw)) continue;
                int k;
                float wd;
                while (dd3_pixwalk_next(dp, &pw, &k, &wd)) {
                    const float coef = dd3_coef(GEOM, FAMILY, &g, &w, lpos, j, wd, lz.w);
                    const float mag = mg[k];
                    const float *__restrict__ ssk = ssv + k;
                    // rows meeting each slice of the slab; the first row of
                    // slice q + 1 is found from where slice q stopped
                    int rnext = -1;
#pragma unroll
                    for (int q = 0; q < kZS; q++) {
                        const int s = s0 + q;
                        if (s < Dp) {
                            const float zlo = zb[q], zhi = zb[q + 1];
                            int r;
                            if (rnext < 0) {
                                r = dd3_row_first(GEOM, &w, rz, R, mag, zlo, 0.0f);
                            } else {
                                r = max(rnext - 1, 0);
                                for (int it = 0; it < 64 && r > 0; it++) {
                                    float e0, e1;
                                    dd3_rp(GEOM, &w, mag, rz[2 * (r - 1)], rz[2 * (r - 1) + 1], &e0, &e1);
                                    if (e1 > zlo) r--;
                                    else break;
                                }
                            }
                            for (; r < R; r++) {
                                float e0, e1;
                                dd3_rp(GEOM, &w, mag, rz[2 * r], rz[2 * r + 1], &e0, &e1);
                                if (!(e0 < zhi)) break;
                                const float zw = dd3_cell(fmaxf(lz.x, e0), fminf(lz.y, e1), zlo, zhi);
                                if (zw > 0.0f) {
                                    const float wq = FMUL(zw, coef);
#pragma unroll
                                    for (int b = 0; b < kNB; b++)
                                        if (b < nb) acc[q][b] = fmaf(wq, __ldg(ssk + (size_t)b * per + (size_t)r * C), acc[q][b]);
                                }
                            }
                            rnext = r;
                        }
                    }
                }
            }
        }
        __syncthreads();   // buffer `buf` is refilled by the next iteration's issue
    }
    if (abort_flag) {
        if (tid == 0 && inflight >= 0) dd_mbar_drain(&bar[inflight], ph.parity(inflight));
        if (tid == 0) dd_report_timeout(a.status);
        return;
    }
    if (!active) return;
#pragma unroll
    for (int q = 0; q < kZS; q++) {
        const int s = s0 + q;
        if (s >= Dp) continue;
#pragma unroll
        for (int b = 0; b < kNB; b++) {
            if (b < nb) {
                const size_t o = (((size_t)(b0 + b) * Dp + s) * H + y) * W + x;
                a.out[o] = a.base ? fmaf(a.scale, acc[q][b], a.base[o]) : acc[q][b];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
int geom_of(int scan) {
    return scan == DD_SCAN_CONE_FLAT ? DD_GEOM3_CONE_FLAT : (scan == DD_SCAN_CONE_ARC ? DD_GEOM3_CONE_ARC : DD_GEOM3_SPIRAL);
}

int validate(int scan, int op, const dd_geom3d *g, int B, int V) {
    if (!g) return DD_ERR_INVALID_ARG;
    if (scan < DD_SCAN_CONE_FLAT || scan > DD_SCAN_SPIRAL) return DD_ERR_INVALID_ARG;
    if (op < DD_OP_PROJ || op > DD_OP_BPROJ_TW) return DD_ERR_INVALID_ARG;
    if (g->width <= 0 || g->height <= 0 || g->depth <= 0 || g->num_col <= 0 || g->num_row <= 0 || B <= 0 ||
        V <= 0)
        return DD_ERR_INVALID_ARG;
    const float f[] = {g->pix_x, g->pix_y, g->pix_z, g->col_size, g->row_size, g->iso_source,
                       g->source_detector, g->pix_xshift, g->pix_yshift, g->pix_zshift, g->col_shift,
                       g->row_shift};
    for (float x : f)
        if (!(x == x) || x - x != 0.0f) return DD_ERR_INVALID_ARG;   // NaN / inf
    if (!(g->pix_x > 0 && g->pix_y > 0 && g->pix_z > 0 && g->col_size > 0 && g->row_size > 0))
        return DD_ERR_INVALID_ARG;
    if (!(g->iso_source > 0 && g->source_detector > 0)) return DD_ERR_INVALID_ARG;
    const long long lim = (1LL << 31) - 1;
    if ((long long)g->width * g->height * g->depth * B > lim) return DD_ERR_SIZE_OVERFLOW;
    if ((long long)V * g->num_row * g->num_col * B > lim) return DD_ERR_SIZE_OVERFLOW;
    if (g->width > 8192 || g->height > 8192 || V > 65535 || g->num_row > 65535 || g->num_col > 65535)
        return DD_ERR_SIZE_OVERFLOW;
    // one view's staged data (two buffers) must fit the adjoint's shared memory
    if (adj3_smem(plan_layout(g, V)).total > 200 * 1024) return DD_ERR_SIZE_OVERFLOW;
    return DD_OK;
}

int launch_status() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? DD_OK : DD_ERR_LAUNCH;
}

int plan(int scan, const dd_geom3d *g, const float *angles, const float *sp, int V, void *planp, size_t bytes,
         cudaStream_t st) {
    const PlanLayout P = plan_layout(g, V);
    if (!planp || bytes < P.total) return DD_ERR_WORKSPACE;
    if (!angles || (scan == DD_SCAN_SPIRAL && !sp)) return DD_ERR_INVALID_ARG;
    char *base = (char *)planp;
    const int geom = geom_of(scan);
    dd2::ProfRec *pr = dd2::prof_begin(DD_KERNEL_PLAN, st);
    const dim3 gl((unsigned)((P.nl * P.nch + 127) / 128), (unsigned)V);
    if (geom == DD_GEOM3_CONE_FLAT) {
        k_views3<DD_GEOM3_CONE_FLAT><<<V, kThreads, 0, st>>>(*g, angles, sp, V, base, P);
        k_lines3<DD_GEOM3_CONE_FLAT><<<gl, 128, 0, st>>>(*g, base, P);
    } else if (geom == DD_GEOM3_CONE_ARC) {
        k_views3<DD_GEOM3_CONE_ARC><<<V, kThreads, 0, st>>>(*g, angles, sp, V, base, P);
        k_lines3<DD_GEOM3_CONE_ARC><<<gl, 128, 0, st>>>(*g, base, P);
    } else {
        k_views3<DD_GEOM3_SPIRAL><<<V, kThreads, 0, st>>>(*g, angles, sp, V, base, P);
        k_lines3<DD_GEOM3_SPIRAL><<<gl, 128, 0, st>>>(*g, base, P);
    }
    k_slab_views3<<<P.nslab, 256, 0, st>>>(*g, base, P, V);
    dd2::prof_end(pr, st);
    dd2::count_launches(3);
    return launch_status();
}

template <int GEOM>
int launch_fwd(int family, const Fwd3Args &a, cudaStream_t st) {
    const dim3 grid((unsigned)a.V, (unsigned)((a.g.num_col + kFC - 1) / kFC),
                    (unsigned)(a.nrb * ((a.B + kNB - 1) / kNB)));
    dd2::ProfRec *pr = dd2::prof_begin(DD_KERNEL_FORWARD, st);
    if (family == 0) k_fwd3<GEOM, 0><<<grid, kFwdThreads3, 0, st>>>(a);
    else if (family == 1) k_fwd3<GEOM, 1><<<grid, kFwdThreads3, 0, st>>>(a);
    else k_fwd3<GEOM, 2><<<grid, kFwdThreads3, 0, st>>>(a);
    dd2::prof_end(pr, st);
    dd2::count_launches(1);
    return launch_status();
}

template <int GEOM, int FAMILY>
int launch_adj_kernel(const Adj3Args &a, const dim3 &grid, cudaStream_t st) {
    const int smem = adj3_smem(a.P).total;
    if (cudaFuncSetAttribute(k_adj3<GEOM, FAMILY>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return DD_ERR_LAUNCH;
    k_adj3<GEOM, FAMILY><<<grid, kThreads, smem, st>>>(a);
    return DD_OK;
}

template <int GEOM>
int launch_adj(int family, const Adj3Args &a, const float *in, float *ss, cudaStream_t st) {
    const dd_geom3d &g = a.g;
    const dim3 gs((unsigned)((g.num_col + 127) / 128), (unsigned)g.num_row, (unsigned)a.V);
    dd2::ProfRec *pt = dd2::prof_begin(DD_KERNEL_TABLES, st);
    if (family == 0) k_sino3<GEOM, 0><<<gs, 128, 0, st>>>(g, a.plan, a.P, in, ss, a.B, a.V);
    else k_sino3<GEOM, 1><<<gs, 128, 0, st>>>(g, a.plan, a.P, in, ss, a.B, a.V);
    dd2::prof_end(pt, st);
    const int nty = (g.height + kTile - 1) / kTile;
    const dim3 grid((unsigned)(a.ntx * nty), (unsigned)((g.depth + kZS - 1) / kZS), (unsigned)((a.B + kNB - 1) / kNB));
    dd2::ProfRec *pr = dd2::prof_begin(DD_KERNEL_ADJOINT, st);
    int rc;
    if (family == 0) rc = launch_adj_kernel<GEOM, 0>(a, grid, st);
    else if (family == 1) rc = launch_adj_kernel<GEOM, 1>(a, grid, st);
    else rc = launch_adj_kernel<GEOM, 2>(a, grid, st);
    dd2::prof_end(pr, st);
    if (rc != DD_OK) return rc;
    dd2::count_launches(2);
    return launch_status();
}

int transpose(const dd_geom3d *g, const float *in, float *out, int B, cudaStream_t st) {
    const int np = B * g->depth;
    const dim3 grid((unsigned)((g->width + 31) / 32), (unsigned)((g->height + 31) / 32),
                    (unsigned)(np < 65535 ? np : 65535));
    dd2::ProfRec *pr = dd2::prof_begin(DD_KERNEL_TABLES, st);
    k_transpose3<<<grid, 256, 0, st>>>(in, out, g->width, g->height, np);
    dd2::prof_end(pr, st);
    dd2::count_launches(1);
    return launch_status();
}

// Forward-type operator into `out` (optionally minus `sub`).
int forward(int scan, int op, const dd_geom3d *g, const char *planb, const float *in, float *out,
            const float *sub, int B, int V, char *volT, int *status, cudaStream_t st) {
    const int s1 = transpose(g, in, (float *)volT, B, st);
    if (s1 != DD_OK) return s1;
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    Fwd3Args a;
    a.status = status;
    a.g = *g;
    a.plan = planb;
    a.P = plan_layout(g, V);
    a.vol = in;
    a.volT = (const float *)volT;
    a.out = out;
    a.sub = sub;
    a.B = B;
    a.V = V;
    a.nrb = (g->num_row + kFR * kFwdWarps3 - 1) / (kFR * kFwdWarps3);
    const int fam = op_family(op), geom = geom_of(scan);
    if (geom == DD_GEOM3_CONE_FLAT) return launch_fwd<DD_GEOM3_CONE_FLAT>(fam, a, st);
    if (geom == DD_GEOM3_CONE_ARC) return launch_fwd<DD_GEOM3_CONE_ARC>(fam, a, st);
    return launch_fwd<DD_GEOM3_SPIRAL>(fam, a, st);
}

// Adjoint-type operator: out = value, or out = base + scale * value.
int adjoint(int scan, int op, const dd_geom3d *g, const char *planb, const float *in, float *out,
            const float *basep, float scale, int B, int V, char *ss, int *status, cudaStream_t st) {
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    Adj3Args a;
    a.status = status;
    a.g = *g;
    a.plan = planb;
    a.P = plan_layout(g, V);
    a.ss = (const float *)ss;
    a.out = out;
    a.base = basep;
    a.scale = scale;
    a.B = B;
    a.V = V;
    a.ntx = (g->width + kTile - 1) / kTile;
    const int fam = op_family(op), geom = geom_of(scan);
    if (geom == DD_GEOM3_CONE_FLAT) return launch_adj<DD_GEOM3_CONE_FLAT>(fam, a, in, (float *)ss, st);
    if (geom == DD_GEOM3_CONE_ARC) return launch_adj<DD_GEOM3_CONE_ARC>(fam, a, in, (float *)ss, st);
    return launch_adj<DD_GEOM3_SPIRAL>(fam, a, in, (float *)ss, st);
}

}   // namespace dd3

using namespace dd3;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int dd3d_validate(int scan, int op, const dd_geom3d *g, int batch, int num_view) {
    return validate(scan, op, g, batch, num_view);
}

extern "C" size_t dd3d_plan_bytes(int scan, const dd_geom3d *g, int num_view) {
    (void)scan;
    if (!g || num_view <= 0) return 0;
    return plan_layout(g, num_view).total;
}

extern "C" int dd3d_plan(int scan, const dd_geom3d *g, const float *angles, const float *source_pos, int num_view,
                         void *planp, size_t plan_bytes, dd_stream_t stream) {
    ddtrace::Range tr("dd3d_plan", scan, -1, true);
    const int st = validate(scan, DD_OP_PROJ, g, 1, num_view);
    if (st != DD_OK) return st;
    return plan(scan, g, angles, source_pos, num_view, planp, plan_bytes, (cudaStream_t)stream);
}

extern "C" size_t dd3d_apply_workspace_bytes(int scan, int op, const dd_geom3d *g, int batch, int num_view) {
    (void)scan;
    if (!g || batch <= 0 || num_view <= 0) return 0;
    const bool f = op_is_forward(op);
    return apply_layout(f, !f, g, batch, num_view).total;
}

extern "C" int dd3d_apply_planned(int scan, int op, const dd_geom3d *g, const void *planp, const float *in,
                                  float *out, int batch, int num_view, void *workspace, size_t workspace_bytes,
                                  dd_stream_t stream) {
    ddtrace::Range tr("dd3d_apply_planned", scan, op, true);
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!planp || !in || !out) return DD_ERR_INVALID_ARG;
    const bool f = op_is_forward(op);
    const ApplyLayout A = apply_layout(f, !f, g, batch, num_view);
    if (!workspace || workspace_bytes < A.total) return DD_ERR_WORKSPACE;
    char *wb = (char *)workspace;
    cudaStream_t s = (cudaStream_t)stream;
    int *status = (int *)(wb + A.status);
    if (f) return forward(scan, op, g, (const char *)planp, in, out, nullptr, batch, num_view, wb + A.volT, status, s);
    return adjoint(scan, op, g, (const char *)planp, in, out, nullptr, 0.0f, batch, num_view, wb + A.ss, status, s);
}

extern "C" size_t dd3d_workspace_bytes(int scan, int op, const dd_geom3d *g, int batch, int num_view) {
    if (!g || batch <= 0 || num_view <= 0) return 0;
    return dd3d_plan_bytes(scan, g, num_view) + dd3d_apply_workspace_bytes(scan, op, g, batch, num_view);
}

extern "C" int dd3d_apply(int scan, int op, const dd_geom3d *g, const float *in, float *out, const float *angles,
                          const float *source_pos, int batch, int num_view, void *workspace,
                          size_t workspace_bytes, dd_stream_t stream) {
    ddtrace::Range tr("dd3d_apply", scan, op, true);
    const int st = validate(scan, op, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!in || !out || !angles || (scan == DD_SCAN_SPIRAL && !source_pos)) return DD_ERR_INVALID_ARG;
    const size_t pb = dd3d_plan_bytes(scan, g, num_view);
    if (!workspace || workspace_bytes < dd3d_workspace_bytes(scan, op, g, batch, num_view)) return DD_ERR_WORKSPACE;
    const int s1 = plan(scan, g, angles, source_pos, num_view, workspace, pb, (cudaStream_t)stream);
    if (s1 != DD_OK) return s1;
    return dd3d_apply_planned(scan, op, g, workspace, in, out, batch, num_view, (char *)workspace + pb,
                              workspace_bytes - pb, stream);
}

extern "C" size_t dd3d_dc_workspace_bytes(int scan, const dd_geom3d *g, int batch, int num_view) {
    (void)scan;
    if (!g || batch <= 0 || num_view <= 0) return 0;
    return apply_layout(true, true, g, batch, num_view).total;
}

extern "C" int dd3d_dc_step(int scan, const dd_geom3d *g, const void *planp, float *x, const float *y, float *resid,
                            float eta, int batch, int num_view, void *workspace, size_t workspace_bytes,
                            dd_stream_t stream) {
    ddtrace::Range tr("dd3d_dc_step", scan, -1, true);
    const int st = validate(scan, DD_OP_PROJ, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!planp || !x || !y || !resid) return DD_ERR_INVALID_ARG;
    const ApplyLayout A = apply_layout(true, true, g, batch, num_view);
    if (!workspace || workspace_bytes < A.total) return DD_ERR_WORKSPACE;
    char *wb = (char *)workspace;
    cudaStream_t s = (cudaStream_t)stream;
    const char *pb = (const char *)planp;
    int *status = (int *)(wb + A.status);
    const int s1 = forward(scan, DD_OP_PROJ, g, pb, x, resid, y, batch, num_view, wb + A.volT, status, s);
    if (s1 != DD_OK) return s1;
    return adjoint(scan, DD_OP_PROJ_T, g, pb, resid, x, x, -eta, batch, num_view, wb + A.ss, status + 1, s);
}

extern "C" int dd3d_status(int scan, int op, const dd_geom3d *g, int batch, int num_view, const void *workspace,
                           int *status) {
    if (validate(scan, op, g, batch, num_view) != DD_OK || !workspace || !status) return DD_ERR_INVALID_ARG;
    const bool f = op_is_forward(op);
    const size_t off = dd3d_plan_bytes(scan, g, num_view) + apply_layout(f, !f, g, batch, num_view).status;
    if (cudaMemcpy(status, (const char *)workspace + off, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return DD_ERR_LAUNCH;
    return DD_OK;
}

extern "C" int dd3d_planned_status(int op, const dd_geom3d *g, int batch, int num_view, const void *workspace,
                                   int *status) {
    if (!g || batch <= 0 || num_view <= 0 || !workspace || !status) return DD_ERR_INVALID_ARG;
    const bool f = op_is_forward(op);
    const size_t off = apply_layout(f, !f, g, batch, num_view).status;
    if (cudaMemcpy(status, (const char *)workspace + off, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return DD_ERR_LAUNCH;
    return DD_OK;
}

int dd3_set_sink(int *sink) { return dd_set_status_sink_tu(sink); }

// named entries (RadonTorch.cpp:1395-1414)
#define DD_NAMED3(name, scan, op)                                                                          \
    extern "C" int dd_##name(const dd_geom3d *g, const float *in, float *out, const float *angles,           \
                             const float *source_pos, int batch, int num_view, void *workspace,             \
                             size_t workspace_bytes, dd_stream_t stream) {                                  \
        return dd3d_apply(scan, op, g, in, out, angles, source_pos, batch, num_view, workspace,            \
                          workspace_bytes, stream);                                                         \
    }
DD_NAMED3(ProjConeFlatDis3d, DD_SCAN_CONE_FLAT, DD_OP_PROJ)
DD_NAMED3(ProjTransConeFlatDis3d, DD_SCAN_CONE_FLAT, DD_OP_PROJ_T)
DD_NAMED3(BackProjConeFlatDis3d, DD_SCAN_CONE_FLAT, DD_OP_BPROJ)
DD_NAMED3(BackProjTransConeFlatDis3d, DD_SCAN_CONE_FLAT, DD_OP_BPROJ_T)
DD_NAMED3(BackProjWeightedConeFlatDis3d, DD_SCAN_CONE_FLAT, DD_OP_BPROJ_W)
DD_NAMED3(BackProjTransWeightedConeFlatDis3d, DD_SCAN_CONE_FLAT, DD_OP_BPROJ_TW)
DD_NAMED3(ProjConeArcDis3d, DD_SCAN_CONE_ARC, DD_OP_PROJ)
DD_NAMED3(ProjTransConeArcDis3d, DD_SCAN_CONE_ARC, DD_OP_PROJ_T)
DD_NAMED3(BackProjConeArcDis3d, DD_SCAN_CONE_ARC, DD_OP_BPROJ)
DD_NAMED3(BackProjTransConeArcDis3d, DD_SCAN_CONE_ARC, DD_OP_BPROJ_T)
DD_NAMED3(BackProjWeightedConeArcDis3d, DD_SCAN_CONE_ARC, DD_OP_BPROJ_W)
DD_NAMED3(BackProjTransWeightedConeArcDis3d, DD_SCAN_CONE_ARC, DD_OP_BPROJ_TW)
DD_NAMED3(ProjSpiralDis3d, DD_SCAN_SPIRAL, DD_OP_PROJ)
DD_NAMED3(ProjTransSpiralDis3d, DD_SCAN_SPIRAL, DD_OP_PROJ_T)
DD_NAMED3(BackProjSpiralDis3d, DD_SCAN_SPIRAL, DD_OP_BPROJ)
DD_NAMED3(BackProjTransSpiralDis3d, DD_SCAN_SPIRAL, DD_OP_BPROJ_T)
DD_NAMED3(BackProjWeightedSpiralDis3d, DD_SCAN_SPIRAL, DD_OP_BPROJ_W)
DD_NAMED3(BackProjTransWeightedSpiralDis3d, DD_SCAN_SPIRAL, DD_OP_BPROJ_TW)
#undef DD_NAMED3
