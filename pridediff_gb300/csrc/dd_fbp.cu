// FBP detector-row filtering with the cosine weight fused.
//
// deeprecon's filtered_backprojection (projector.py:192-213 for 2-D fan and
// parallel beams, :368-390 for cone beams, :554-563 for spirals) weights the
// sinogram and filters every detector row with a 2D - 1 tap kernel:
//
//     nn.functional.conv2d(sino * weight, filter, padding=(0, D - 1))
//
// (conv3d for the 3-D geometries), i.e. the cross-correlation
//
//     out[i][k] = sum_n taps[n - k + D - 1] * (weight[i % wrows][n] * in[i][n])
//
// over the D bins n of row i, before the weighted DD back-projection.  One
// kernel does both: a CTA stages the taps and the weighted rows of kRows rows
// in shared memory and each thread accumulates kOut adjacent outputs of every
// row, sliding a register window over the taps, so that one tap load and kRows
// broadcast loads feed kRows * kOut FMAs.  The products are rounded once as
// the reference's `sino * weight` is; the sums run in FP32 in bin order.
#include <cuda_runtime.h>

#include "../../include/pridediff_dd.h"
#include "dd_trace.h"

namespace dd2 {
struct ProfRec;
ProfRec *prof_begin(int kind, cudaStream_t st);
void prof_end(ProfRec *r, cudaStream_t st);
void count_launches(int n);
}   // namespace dd2

namespace ddfbp {

constexpr int kThreads = 256;
constexpr int kRows = 4;   // rows per CTA (the taps are staged once for them)
constexpr int kOut = 4;    // adjacent outputs per thread and row

__host__ __device__ inline int taps_stride(int D) { return (2 * D - 1 + 3) & ~3; }

inline size_t smem_bytes(int D) { return sizeof(float) * ((size_t)taps_stride(D) + (size_t)kRows * D); }

// weight == nullptr: unit weight.
__global__ void __launch_bounds__(kThreads)
k_fbp_filter(const float *__restrict__ in, float *__restrict__ out, const float *__restrict__ weight, int wrows,
             const float *__restrict__ taps, long long rows, int D) {
    extern __shared__ float sm[];
    float *st = sm;                      // taps, 2D - 1
    float *sx = sm + taps_stride(D);     // kRows weighted rows of D bins
    const int tid = threadIdx.x;
    const long long row0 = (long long)blockIdx.x * kRows;
    const int nr = (int)min((long long)kRows, rows - row0);
    for (int i = tid; i < 2 * D - 1; i += kThreads) st[i] = taps[i];
    for (int r = 0; r < kRows; r++) {
        const float *src = in + (row0 + r) * D;
        const float *wr = weight ? weight + ((row0 + r) % wrows) * D : nullptr;
        for (int n = tid; n < D; n += kThreads)
            sx[r * D + n] = (r < nr) ? (wr ? __fmul_rn(src[n], wr[n]) : src[n]) : 0.0f;
    }
    __syncthreads();
    for (int k0 = tid * kOut; k0 < D; k0 += kThreads * kOut) {
        float acc[kRows][kOut];
#pragma unroll
        for (int r = 0; r < kRows; r++)
#pragma unroll
            for (int i = 0; i < kOut; i++) acc[r][i] = 0.0f;
        // output k0 + i at bin n needs taps[n - k0 - i + D - 1] (in 0 .. 2D - 2
        // for the outputs k0 + i < D; the window entries of outputs past the
        // row end start at zero and are never written); window t[i] holds it
        // and slides by one entry per bin.
        float t[kOut];
#pragma unroll
        for (int i = 0; i < kOut; i++) {
            const int ti = D - 1 - k0 - i;   // tap index at n = 0 (negative: not yet reached)
            t[i] = (ti >= 0) ? st[ti] : 0.0f;
        }
        for (int n = 0; n < D; n++) {
            float xv[kRows];
#pragma unroll
            for (int r = 0; r < kRows; r++) xv[r] = sx[r * D + n];
#pragma unroll
            for (int r = 0; r < kRows; r++)
#pragma unroll
                for (int i = 0; i < kOut; i++) acc[r][i] = fmaf(t[i], xv[r], acc[r][i]);
            // slide: at n + 1 output k0 + i needs taps[n + 1 - k0 - i + D - 1],
            // which output k0 + i - 1 used at n
#pragma unroll
            for (int i = kOut - 1; i > 0; i--) t[i] = t[i - 1];
            const int t0 = n + 1 - k0 + D - 1;   // <= 2D - 2 for n + 1 < D
            t[0] = (n + 1 < D) ? st[t0] : 0.0f;
        }
#pragma unroll
        for (int r = 0; r < kRows; r++) {
            if (r >= nr) break;
#pragma unroll
            for (int i = 0; i < kOut; i++)
                if (k0 + i < D) out[(row0 + r) * D + k0 + i] = acc[r][i];
        }
    }
}

}   // namespace ddfbp

using namespace ddfbp;

extern "C" int dd_fbp_filter(const float *in, float *out, const float *weight, int wrows, const float *taps,
                             long long rows, int num_det, dd_stream_t stream) {
    ddtrace::Range tr("dd_fbp_filter");
    if (!in || !out || !taps || rows <= 0 || num_det <= 0 || (weight && wrows <= 0)) return DD_ERR_INVALID_ARG;
    if (num_det > 8192 || (rows + kRows - 1) / kRows > 2147483647LL) return DD_ERR_SIZE_OVERFLOW;
    const size_t sb = smem_bytes(num_det);
    if (cudaFuncSetAttribute(k_fbp_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb) != cudaSuccess)
        return DD_ERR_LAUNCH;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((rows + kRows - 1) / kRows);
    dd2::ProfRec *pr = dd2::prof_begin(DD_KERNEL_FILTER, st);
    k_fbp_filter<<<grid, kThreads, sb, st>>>(in, out, weight, weight ? wrows : 1, taps, rows, num_det);
    dd2::prof_end(pr, st);
    dd2::count_launches(1);
    return cudaGetLastError() == cudaSuccess ? DD_OK : DD_ERR_LAUNCH;
}
