// Host model of the 2-D CUDA kernels (test infrastructure).
//
// Compiles the same geometry header the kernels use (dd_geom2d.cuh, host
// branch of its rounding macros) and evaluates the forward (detector-gather)
// and adjoint (pixel-gather) integral forms exactly as k_fwd / k_adj in
// pridediff_gb300/csrc/dd2d.cu do, one line at a time, in FP32 with fmaf.
// The CPU tests compare it with deeprecon's own CPU projectors: this checks
// the bit-exact geometry replication, the drift-piece model and the integral
// formulas without a GPU.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared dd_model2d.cpp
#include <cmath>
#include <cstring>
#include <vector>

#include "../../pridediff_gb300/csrc/dd_geom2d.cuh"

namespace {

struct F2 {
    float S, x;
};

// K_p of every piece (sequential form of piece_K).
std::vector<float> piece_K(const DdLine &L, const F2 *tab) {
    std::vector<float> K(L.h.npiece);
    float run = 0.0f;
    for (int p = 0; p < L.h.npiece; p++) {
        const DdPiece P = L.p[p];
        const int first = (p == 0) ? L.h.i0 : L.p[p - 1].gb + 1;
        const float fv = FADD(P.Q, FMUL((float)(first - P.gb), P.dl));
        const float prevQ = (p == 0) ? L.h.bound0 : L.p[p - 1].Q;
        const float prevdl = (p == 0) ? 0.0f : L.p[p - 1].dl;
        const float term = std::fmaf(prevdl, tab[first].S,
                                     std::fmaf(tab[first].x, fv - prevQ, -P.dl * tab[first + 1].S));
        run += term;
        K[p] = run;
    }
    return K;
}

float integral(const DdLine &L, const std::vector<float> &K, const F2 *tab, float u) {
    int p, j;
    float r;
    dd_locate(&L, u, &p, &j, &r);
    return std::fmaf(r, tab[j].x, std::fmaf(L.p[p].dl, tab[j].S, K[p]));
}

std::vector<F2> prefix(const float *x, int n, int stride) {
    std::vector<F2> t(n + 1);
    double run = 0.0;
    for (int i = 0; i < n; i++) {
        const float v = x[(long)i * stride];
        t[i] = {(float)run, v};
        run += v;
    }
    t[n] = {(float)run, 0.0f};
    return t;
}

int det_index_fan(int geom, const dd_geom2d &g, const DdView2 &vw, float view, float u) {
    const int D = g.num_det;
    float kf;
    if (geom == DD_GEOM_FLAT) {
        const float R = g.iso_source;
        const float vds = FMUL(FDIV(R, g.source_detector), g.det_size);
        const float vbs = FMUL(FDIV(R, g.source_detector), g.bin_shift);
        const float t = vw.xb ? R * u * vw.c / (R + u * vw.s) : R * u * vw.s / (R - u * vw.c);
        const float q = (t - vbs) / vds;
        kf = vw.flip ? (float)D * 0.5f - q : q + (float)D * 0.5f;
    } else {
        float ang = vw.xb ? std::atan2(u - vw.srcx, vw.srcy)
                          : 1.5707963267948966f - std::atan((u - vw.srcy) / vw.srcx);
        const float base = view + g.bin_shift;
        ang += 3.14159265358979f * std::rint((base - ang) * 0.3183098861837907f);
        const float q = (ang - base) / g.det_size;
        kf = vw.flip ? (float)D * 0.5f - q : q + (float)D * 0.5f;
    }
    int k = (int)std::floor(kf);
    return k < 0 ? 0 : (k > D - 1 ? D - 1 : k);
}

}  // namespace

// op: 0 proj, 1 proj_t, 2 bproj, 3 bproj_t, 4 bproj_w, 5 bproj_tw.  scan: 0 para, 1 flat, 2 arc.
// in/out: reference layouts, batch B.  Returns 0 on success.
extern "C" int model_apply2d(int scan, int op, const dd_geom2d *gp, const float *in, float *out,
                             const float *angles, int B, int V) {
    const dd_geom2d g = *gp;
    const int geom = scan;
    const int W = g.width, H = g.height, D = g.num_det;
    const bool fwd = (op == 0 || op == 3 || op == 5);
    if (fwd) std::memset(out, 0, sizeof(float) * (size_t)B * V * D);
    else std::memset(out, 0, sizeof(float) * (size_t)B * H * W);
    std::vector<float> dp(D + 1), bc(D + 1);
    DdLine L, Ld;
    for (int v = 0; v < V; v++) {
        const float view = angles[v];
        DdView2 vw;
        dd_view2_setup(geom, &g, view, &vw, dp.data(), bc.data());
        const int nline = vw.xb ? H : W, npix = vw.xb ? W : H;
        const float para_beta = vw.xb ? FDIV(g.pix_y, g.det_size) : FDIV(g.pix_x, g.det_size);
        for (int b = 0; b < B; b++) {
            std::vector<float> acc(fwd ? D : 0, 0.0f);
            // sorted detector row and its integral table (adjoint)
            std::vector<F2> dt;
            if (!fwd) {
                std::vector<float> gk(D);
                const float *s = in + ((size_t)b * V + v) * D;
                dt.resize(D + 1);
                double run = 0.0;
                for (int k = 0; k < D; k++) {
                    const float sv = s[vw.flip ? D - 1 - k : k];
                    float gg;
                    double w;
                    if (geom == DD_GEOM_PARA) {
                        gg = (op == 1) ? sv * para_beta : sv;
                        w = 1.0;
                    } else {
                        gg = (op == 1) ? sv * bc[k] : sv;
                        w = (double)(dp[k + 1] - dp[k]);
                    }
                    dt[k] = {(float)run, gg};
                    run += (double)gg * w;
                }
                dt[D] = {(float)run, 0.0f};
            }
            for (int line = 0; line < nline; line++) {
                dd_line2_setup(geom, &g, view, &vw, dp.data(), line, &L,
                               geom == DD_GEOM_PARA ? &Ld : nullptr);
                if (L.h.npiece == 0) continue;
                const float bound0 = L.h.bound0, endv = L.h.endv;
                const int idet0 = L.h.idet0;
                if (fwd) {
                    const float *img = in + (size_t)b * H * W;
                    std::vector<F2> tab = vw.xb ? prefix(img + (size_t)line * W, W, 1)
                                                : prefix(img + (size_t)(H - 1) * W + line, H, -W);
                    if (op == 5) {
                        // FBP-weighted transpose: weight every pixel at this view, rebuild the prefix
                        const float lpos = vw.xb
                            ? (float)(((double)H / 2.0 - line - 0.5) * (double)g.pix_y + (double)g.pix_yshift)
                            : (float)(((double)line - W / 2.0 + 0.5) * (double)g.pix_x + (double)g.pix_xshift);
                        float run = 0.0f;
                        for (int i = 0; i < npix; i++) {
                            float pcx, pcy;
                            if (vw.xb) {
                                pcx = (float)(((double)i + 0.5) * (double)g.pix_x + (double)vw.axis0);
                                pcy = lpos;
                            } else {
                                pcx = lpos;
                                pcy = (float)(((double)i + 0.5) * (double)g.pix_y + (double)vw.axis0);
                            }
                            const float w = (geom == DD_GEOM_ARC) ? 1.0f / dd_cw_arc(vw.srcx, vw.srcy, pcx, pcy)
                                                                  : dd_cw_flat(vw.srcx, vw.srcy, pcx, pcy, g.iso_source);
                            const float y = tab[i].x * w;
                            tab[i] = {run, y};
                            run += y;
                        }
                        tab[npix] = {run, 0.0f};
                    }
                    const std::vector<float> K = piece_K(L, tab.data());
                    const float scale = (op == 0) ? 1.0f : L.h.alpha;
                    float prev = 0.0f;
                    for (int kb = 0; kb <= D; kb++) {
                        float u;
                        if (kb <= idet0) u = bound0;
                        else if (geom == DD_GEOM_PARA) {
                            const int idx = kb - 1;
                            const float est = Ld.p[0].Q + (float)(idx - Ld.p[0].gb) * Ld.p[0].dl;
                            u = Ld.h.npiece > 0 ? dd_boundary(&Ld, idx, est) : bound0;
                        } else u = dp[kb];
                        u = std::fmin(std::fmax(u, bound0), endv);
                        const float f = integral(L, K, tab.data(), u);
                        if (kb > 0) acc[kb - 1] = std::fmaf(scale, f - prev, acc[kb - 1]);
                        prev = f;
                    }
                } else {
                    std::vector<float> Kd;
                    if (geom == DD_GEOM_PARA && Ld.h.npiece > 0) Kd = piece_K(Ld, dt.data());
                    auto Hval = [&](float u) -> float {
                        if (geom == DD_GEOM_PARA) {
                            if (Ld.h.npiece == 0) return 0.0f;
                            const float uu = std::fmin(std::fmax(u, bound0), Ld.h.endv);
                            return integral(Ld, Kd, dt.data(), uu);
                        }
                        const float uu = std::fmin(std::fmax(u, bound0), dp[D]);
                        int k = det_index_fan(geom, g, vw, view, uu);
                        // one-step correction against the exact boundary table
                        if (k > 0 && uu < dp[k]) k--;
                        else if (k < D - 1 && uu >= dp[k + 1]) k++;
                        if (k < idet0) k = idet0;
                        return std::fmaf(uu - dp[k], dt[k].x, dt[k].S);
                    };
                    const float alpha = (op == 1) ? 1.0f : L.h.alpha;
                    float hprev = Hval(bound0);
                    for (int i = L.h.i0; i < npix; i++) {
                        const float est = L.p[0].Q + (float)(i - L.p[0].gb) * L.p[0].dl;
                        const float up = dd_boundary(&L, i, est);
                        const float hu = Hval(up);
                        float wgt = 1.0f;
                        if (op == 4) {
                            float pcx, pcy;
                            if (vw.xb) {
                                pcx = (float)(((double)i + 0.5) * (double)g.pix_x + (double)vw.axis0);
                                pcy = (float)(((double)H / 2.0 - line - 0.5) * (double)g.pix_y + (double)g.pix_yshift);
                            } else {
                                pcx = (float)(((double)line - W / 2.0 + 0.5) * (double)g.pix_x + (double)g.pix_xshift);
                                pcy = (float)(((double)i + 0.5) * (double)g.pix_y + (double)vw.axis0);
                            }
                            wgt = (geom == DD_GEOM_ARC) ? 1.0f / dd_cw_arc(vw.srcx, vw.srcy, pcx, pcy)
                                                        : dd_cw_flat(vw.srcx, vw.srcy, pcx, pcy, g.iso_source);
                        }
                        const float val = alpha * (hu - hprev) * wgt;
                        const size_t o = vw.xb ? ((size_t)b * H + line) * W + i
                                               : ((size_t)b * H + (H - 1 - i)) * W + line;
                        out[o] += val;
                        hprev = hu;
                    }
                }
            }
            if (fwd) {
                for (int k = 0; k < D; k++) {
                    float beta = 1.0f;
                    if (op == 0) beta = (geom == DD_GEOM_PARA) ? para_beta : bc[k];
                    out[((size_t)b * V + v) * D + (vw.flip ? D - 1 - k : k)] = acc[k] * beta;
                }
            }
        }
    }
    return 0;
}

// Piece-model check: boundaries i0..nend-1 produced by the reference's FP32
// recurrence b_{i+1} = fl(b_i + pint) from b_{i0} = v0, against the piece
// model.  Returns how many differ; *npiece receives the piece count.
extern "C" int model_check_pieces(float v0, float pint, int i0, int nend, int *npiece, int *flags,
                                  float *maxdev_ulp) {
    DdLine L;
    int fl = 0;
    L.h.i0 = i0;
    L.h.nend = nend;
    L.h.bound0 = v0 - pint;
    L.h.npiece = dd_build_pieces(v0, pint, i0, nend, L.p, &fl);
    dd_build_slots(L.p, L.h.npiece, L.slot);
    *npiece = L.h.npiece;
    *flags = fl;
    int bad = 0;
    float worst = 0.0f;
    float x = v0;
    for (int i = i0; i < nend; i++) {
        const float est = v0 + (float)(i - i0) * pint;
        const float m = dd_boundary(&L, i, est);
        if (m != x) {
            bad++;
            const float ulp = std::nextafter(std::fabs(x), INFINITY) - std::fabs(x);
            const float dev = std::fabs(m - x) / ulp;
            if (dev > worst) worst = dev;
        }
        // locate() must map the boundary value back to the pixel above it
        int p, j;
        float r;
        dd_locate(&L, x, &p, &j, &r);
        if (!(j == i + 1 || (j == i && r >= 0.0f) || (i + 1 == nend && j == nend))) bad += 1000000;
        x = x + pint;
    }
    *maxdev_ulp = worst;
    return bad;
}

// System matrix through the kernels' line walk (dd_line2_sysmat), view by
// view and line by line like deeprecon's builders.  With rows == NULL only
// the number of entries is returned.
extern "C" long long model_sysmatrix2d(int scan, const dd_geom2d *gp, const float *angles, int V, long long *rows,
                                       long long *cols, float *vals) {
    const dd_geom2d g = *gp;
    const int geom = scan;
    const int D = g.num_det, nl = g.height > g.width ? g.height : g.width;
    std::vector<float> dp(D + 1), bc(D + 1);
    long long n = 0;
    for (int v = 0; v < V; v++) {
        DdView2 vw;
        dd_view2_setup(geom, &g, angles[v], &vw, dp.data(), bc.data());
        for (int line = 0; line < nl; line++)
            n += dd_line2_sysmat(geom, &g, angles[v], &vw, dp.data(), bc.data(), v, line, rows ? rows + n : nullptr,
                                 rows ? cols + n : nullptr, rows ? vals + n : nullptr);
    }
    return n;
}
