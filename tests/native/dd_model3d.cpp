// Host model of the 3-D CUDA kernels (test infrastructure).
//
// Compiles the geometry header the kernels use (dd_geom3d.cuh, host branch
// of its rounding macros) and evaluates the forward-type operators by
// column-segment walks (as k_fwd3 does per detector bin) and the
// adjoint-type operators by pixel-segment walks with the row-candidate
// search (as k_adj3 does per voxel).  The CPU tests compare it with the 3-D
// oracle, checking the geometry replication, the per-block drift records and
// the segment formulas without a GPU.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared dd_model3d.cpp
#include <cmath>
#include <cstring>
#include <vector>

#include "../../pridediff_gb300/csrc/dd_geom3d.cuh"

namespace {

struct Plan3 {
    int V, nl, nch;
    std::vector<DdView3> views;
    std::vector<float> dp, mag, rowz, linez;
    std::vector<DdLine> lines;
};

void build_plan(int geom, const dd_geom3d *g, const float *angles, const float *sp, int V, Plan3 &P) {
    const int C = g->num_col, R = g->num_row;
    P.V = V;
    P.nl = g->height > g->width ? g->height : g->width;
    P.nch = (C + DD3_CHUNK - 1) / DD3_CHUNK;
    P.views.resize(V);
    P.dp.resize((size_t)V * (C + 1));
    P.mag.resize((size_t)V * C);
    P.rowz.resize((size_t)V * R * 2);
    P.linez.resize((size_t)V * P.nl * 4);
    P.lines.resize((size_t)V * P.nl * P.nch);
    for (int v = 0; v < V; v++) {
        float sp4[4] = {0, 0, 0, 0};
        if (sp)
            for (int i = 0; i < 4; i++) sp4[i] = sp[(size_t)i * V + v];
        DdView3 &w = P.views[v];
        dd3_view_scalars(geom, g, angles[v], sp4, &w);
        float *dp = &P.dp[(size_t)v * (C + 1)];
        for (int k = 0; k <= C; k++) dp[k] = dd3_col_boundary(geom, g, &w, k);
        float mn = 1e30f, mx = -1e30f;
        for (int k = 0; k < C; k++) {
            const float m = dd3_col_mag(geom, g, &w, k);
            P.mag[(size_t)v * C + k] = m;
            mn = m < mn ? m : mn;
            mx = m > mx ? m : mx;
        }
        w.magmin = mn;
        w.magmax = mx;
        float *rz = &P.rowz[(size_t)v * R * 2];
        for (int r = 0; r < R; r++) dd3_row_z(geom, g, &w, r, &rz[2 * r], &rz[2 * r + 1]);
        w.rzA = rz[0];
        w.rzB = (R > 1) ? (rz[2 * (R - 1)] - rz[0]) / (float)(R - 1) : rz[1] - rz[0];
        const int nline = w.xb ? g->height : g->width;
        for (int l = 0; l < nline; l++)
            for (int cc = 0; cc < P.nch; cc++)
                dd3_line_setup(geom, g, &w, dp, l, cc, &P.linez[((size_t)v * P.nl + l) * 4],
                               &P.lines[((size_t)v * P.nl + l) * P.nch + cc]);
    }
}

inline size_t vox_index(const dd_geom3d *g, const DdView3 &w, int s, int line, int j) {
    const int W = g->width, H = g->height;
    return w.xb ? ((size_t)s * H + line) * W + j : ((size_t)s * H + (H - 1 - j)) * W + line;
}

}  // namespace

extern "C" int model_apply3d(int geom, int op, const dd_geom3d *g, const float *angles, const float *sp,
                             const float *in, float *out, int B, int V) {
    const int W = g->width, H = g->height, Dp = g->depth, C = g->num_col, R = g->num_row;
    Plan3 P;
    build_plan(geom, g, angles, sp, V, P);
    const bool fwd = (op == DD_OP_PROJ || op == DD_OP_BPROJ_T || op == DD_OP_BPROJ_TW);
    const int family = (op == DD_OP_PROJ || op == DD_OP_PROJ_T) ? 0 : (op == DD_OP_BPROJ_W || op == DD_OP_BPROJ_TW) ? 2 : 1;
    const size_t vox_b = (size_t)W * H * Dp, det_b = (size_t)V * R * C;
    if (fwd) {
        for (int b = 0; b < B; b++)
            for (int v = 0; v < V; v++) {
                const DdView3 &w = P.views[v];
                const float *dp = &P.dp[(size_t)v * (C + 1)];
                const float *rz = &P.rowz[(size_t)v * R * 2];
                const int nline = w.xb ? H : W;
                for (int r = 0; r < R; r++)
                    for (int k = 0; k < C; k++) {
                        const int cc = k / DD3_CHUNK, kk = k - cc * DD3_CHUNK;
                        const float mag = P.mag[(size_t)v * C + k];
                        float rp0, rp1;
                        dd3_rp(geom, &w, mag, rz[2 * r], rz[2 * r + 1], &rp0, &rp1);
                        float acc = 0.0f;
                        for (int l = 0; l < nline; l++) {
                            const float *lz = &P.linez[((size_t)v * P.nl + l) * 4];
                            const float bz0 = lz[0] > rp0 ? lz[0] : rp0, bz1 = lz[1] < rp1 ? lz[1] : rp1;
                            if (!(bz0 < bz1)) continue;
                            const DdLine &L = P.lines[((size_t)v * P.nl + l) * P.nch + cc];
                            DdColWalk cw;
                            if (!dd3_colwalk_init(&L, dp, k, kk, &cw)) continue;
                            const float lpos = dd3_line_pos(g, &w, l);
                            int j;
                            float wd;
                            while (dd3_colwalk_next(&L, &cw, &j, &wd)) {
                                const float coef = dd3_coef(geom, family, g, &w, lpos, j, wd, lz[3]);
                                for (int s = dd3_slice_first(bz0, lz[0], lz[2]); s < Dp; s++) {
                                    const float zlo = dd3_zb(lz[0], lz[2], s);
                                    if (!(zlo < bz1)) break;
                                    const float zw = dd3_cell(bz0, bz1, zlo, dd3_zb(lz[0], lz[2], s + 1));
                                    if (zw > 0.0f)
                                        acc = std::fmaf(FMUL(zw, coef), in[b * vox_b + vox_index(g, w, s, l, j)], acc);
                                }
                            }
                        }
                        const float scale = (family == 0) ? dd3_proj_scale(g, &w, dp[k], dp[k + 1], rp0, rp1) : w.bp_scale;
                        const int ko = w.flip ? C - 1 - k : k;
                        out[b * det_b + ((size_t)v * R + r) * C + ko] = FMUL(acc, scale);
                    }
            }
        return 0;
    }
    // adjoint-type: scaled sinogram indexed by sorted column, then voxel gathers
    std::vector<float> ss((size_t)B * det_b);
    for (int b = 0; b < B; b++)
        for (int v = 0; v < V; v++) {
            const DdView3 &w = P.views[v];
            const float *dp = &P.dp[(size_t)v * (C + 1)];
            const float *rz = &P.rowz[(size_t)v * R * 2];
            for (int r = 0; r < R; r++)
                for (int k = 0; k < C; k++) {
                    float scale = w.bp_scale;
                    if (family == 0) {
                        float rp0, rp1;
                        dd3_rp(geom, &w, P.mag[(size_t)v * C + k], rz[2 * r], rz[2 * r + 1], &rp0, &rp1);
                        scale = dd3_proj_scale(g, &w, dp[k], dp[k + 1], rp0, rp1);
                    }
                    const int ko = w.flip ? C - 1 - k : k;
                    ss[b * det_b + ((size_t)v * R + r) * C + k] = FMUL(in[b * det_b + ((size_t)v * R + r) * C + ko], scale);
                }
        }
    for (int b = 0; b < B; b++)
        for (int s = 0; s < Dp; s++)
            for (int y = 0; y < H; y++)
                for (int x = 0; x < W; x++) {
                    float acc = 0.0f;
                    for (int v = 0; v < V; v++) {
                        const DdView3 &w = P.views[v];
                        const float *dp = &P.dp[(size_t)v * (C + 1)];
                        const float *rz = &P.rowz[(size_t)v * R * 2];
                        const int line = w.xb ? y : x;
                        const int j = w.xb ? x : H - 1 - y;
                        const float *lz = &P.linez[((size_t)v * P.nl + line) * 4];
                        const float lpos = dd3_line_pos(g, &w, line);
                        const float zlo = dd3_zb(lz[0], lz[2], s), zhi = dd3_zb(lz[0], lz[2], s + 1);
                        for (int cc = 0; cc < P.nch; cc++) {
                            const DdLine &L = P.lines[((size_t)v * P.nl + line) * P.nch + cc];
                            DdPixWalk pw;
                            if (!dd3_pixwalk_init(geom, g, &w, &L, dp, cc, j, &pw)) continue;
                            int k;
                            float wd;
                            while (dd3_pixwalk_next(dp, &pw, &k, &wd)) {
                                const float coef = dd3_coef(geom, family, g, &w, lpos, j, wd, lz[3]);
                                const float mag = P.mag[(size_t)v * C + k];
                                for (int r = dd3_row_first(geom, &w, rz, R, mag, zlo, 0.0f); r < R; r++) {
                                    float rp0, rp1;
                                    dd3_rp(geom, &w, mag, rz[2 * r], rz[2 * r + 1], &rp0, &rp1);
                                    if (!(rp0 < zhi)) break;
                                    const float bz0 = lz[0] > rp0 ? lz[0] : rp0, bz1 = lz[1] < rp1 ? lz[1] : rp1;
                                    const float zw = dd3_cell(bz0, bz1, zlo, zhi);
                                    if (zw > 0.0f)
                                        acc = std::fmaf(FMUL(zw, coef), ss[b * det_b + ((size_t)v * R + r) * C + k], acc);
                                }
                            }
                        }
                    }
                    out[b * vox_b + ((size_t)s * H + y) * W + x] = acc;
                }
    return 0;
}
