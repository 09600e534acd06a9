// System matrix of a 2-D geometry, built on the GPU: the drop-in for
// deeprecon's GetSysMatrixPara2d / GetSysMatrixFanFlat2d / GetSysMatrixFanArc2d
// (RadonTorch.cpp:1270-1372), which build a COO matrix (V*D x H*W) on the CPU
// with one entry per step of the DD merge walk.
//
// One thread per (view, walked line) runs that walk sequentially with the
// reference's own FP32 recurrences (dd_line2_sysmat in dd_geom2d.cuh), first
// to count its entries, then -- at offsets the caller derives from the counts
// by an exclusive prefix sum -- to write them.  The entries come out in the
// reference's order: view by view, line by line, step by step.
#include "dd2d_kernels.cuh"
#include "dd_trace.h"

namespace dd2 {

__global__ void __launch_bounds__(128)
k_sysmat(int geom, dd_geom2d g, int nl, const DdView2 *__restrict__ views, const float *__restrict__ ang,
         const float *__restrict__ dp, const float *__restrict__ bcoef, long long *__restrict__ counts,
         const long long *__restrict__ offs, long long *__restrict__ rows, long long *__restrict__ cols,
         float *__restrict__ vals) {
    const int line = blockIdx.x * 128 + threadIdx.x, v = blockIdx.y;
    if (line >= nl) return;
    const int D = g.num_det;
    const size_t i = (size_t)v * nl + line;
    const DdView2 vw = views[v];
    const float *dpv = dp + (size_t)v * (D + 1), *bcv = bcoef + (size_t)v * (D + 1);
    if (!offs) {
        counts[i] = dd_line2_sysmat(geom, &g, ang[v], &vw, dpv, bcv, v, line, nullptr, nullptr, nullptr);
        return;
    }
    const long long o = offs[i];
    dd_line2_sysmat(geom, &g, ang[v], &vw, dpv, bcv, v, line, rows + o, cols + o, vals + o);
}

static int sysmat_launch(int scan, const dd_geom2d *g, const void *planp, int V, long long *counts,
                         const long long *offs, long long *rows, long long *cols, float *vals, cudaStream_t st) {
    const int vs = validate(scan, DD_OP_PROJ, g, 1, V);
    if (vs != DD_OK) return vs;
    if (!planp || V > 65535) return !planp ? DD_ERR_INVALID_ARG : DD_ERR_SIZE_OVERFLOW;
    const PlanLayout P = plan_layout(scan, g, V);
    const char *pb = (const char *)planp;
    const dim3 grid((unsigned)((P.nl + 127) / 128), (unsigned)V);
    k_sysmat<<<grid, 128, 0, st>>>(geom_of(scan), *g, P.nl, (const DdView2 *)(pb + P.views),
                                   (const float *)(pb + P.ang), (const float *)(pb + P.dp),
                                   (const float *)(pb + P.bcoef), counts, offs, rows, cols, vals);
    count_launches(1);
    return launch_status();
}

}  // namespace dd2

using namespace dd2;

extern "C" size_t dd2d_sysmatrix_lines(const dd_geom2d *g, int num_view) {
    if (!g || num_view <= 0) return 0;
    return (size_t)num_view * (size_t)(g->height > g->width ? g->height : g->width);
}

extern "C" int dd2d_sysmatrix_count(int scan, const dd_geom2d *g, const void *plan, int num_view, long long *counts,
                                    dd_stream_t stream) {
    ddtrace::Range tr("dd2d_sysmatrix_count", scan, -1, false);
    if (!counts) return DD_ERR_INVALID_ARG;
    return sysmat_launch(scan, g, plan, num_view, counts, nullptr, nullptr, nullptr, nullptr, (cudaStream_t)stream);
}

extern "C" int dd2d_sysmatrix_fill(int scan, const dd_geom2d *g, const void *plan, int num_view,
                                   const long long *offsets, long long *rows, long long *cols, float *vals,
                                   dd_stream_t stream) {
    ddtrace::Range tr("dd2d_sysmatrix_fill", scan, -1, false);
    if (!offsets || !rows || !cols || !vals) return DD_ERR_INVALID_ARG;
    return sysmat_launch(scan, g, plan, num_view, nullptr, offsets, rows, cols, vals, (cudaStream_t)stream);
}
