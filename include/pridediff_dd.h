/*
 * pridediff_dd.h -- C ABI of the GB300 distance-driven (DD) CT projector.
 *
 * Drop-in replacement for the operators of deeprecon's torch extension
 * `radontorch` (deeprecon/interface/RadonTorch.cpp:1375-1418), exposed as a
 * plain C ABI: device pointers, sizes, a host-side geometry record and a CUDA
 * stream.  No torch types cross this boundary; the Python package
 * `pridediff_gb300` binds it with ctypes, and a cgo / JNI / N-API binding
 * would bind the same symbols.
 *
 * Differences from the reference boundary, all deliberate:
 *  - geometry is a host POD (`dd_geom2d`, `dd_geom3d`) holding exactly the
 *    entries of deeprecon's `options` tensor (projector.py:113, :286, :460),
 *    instead of a device tensor read with 11-17 `.item()` syncs per call
 *    (RadonTorch.cpp:19-29);
 *  - work is enqueued on the caller's stream (the reference launches on the
 *    legacy default stream and never checks for errors);
 *  - the library never allocates: scratch comes from the caller through
 *    `workspace` (size from the matching *_workspace_bytes query), so every
 *    call is capturable in a CUDA graph;
 *  - every entry returns a status code (DD_OK = 0) and never aborts.
 *
 * Layouts (all FP32, contiguous, row-major, as in the reference):
 *   2-D image (B, H, W), sinogram (B, V, D)            RadonTorch.cpp:33, :68
 *   3-D volume (B, Dep, H, W), sinogram (B, V, R, C)   RadonTorch.cpp:594, :631
 *   angles (V) on the device; spiral source table (4, V) on the device with
 *   rows [axial position, radius shift, angle shift, axial shift]
 *   (RadonTorch.cpp:1040-1043).
 * B is the product of the reference's batch and channel sizes.
 */
#ifndef PRIDEDIFF_DD_H
#define PRIDEDIFF_DD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without requiring the CUDA headers */
typedef struct CUstream_st *dd_stream_t;

/* status codes */
enum {
    DD_OK = 0,
    DD_ERR_INVALID_ARG = 1,   /* null pointer, non-positive or NaN geometry  */
    DD_ERR_SIZE_OVERFLOW = 2, /* sizes overflow the 32-bit index space      */
    DD_ERR_WORKSPACE = 3,     /* workspace missing or too small             */
    DD_ERR_LAUNCH = 4,        /* a CUDA launch or runtime call failed       */
    DD_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up         */
    DD_ERR_UNSUPPORTED = 6    /* operator not defined for this geometry     */
};

/* scan geometry (projector scan_type) */
enum { DD_SCAN_PARA = 0, DD_SCAN_FLAT = 1, DD_SCAN_ARC = 2 };
enum { DD_SCAN_CONE_FLAT = 0, DD_SCAN_CONE_ARC = 1, DD_SCAN_SPIRAL = 2 };

/* operators (RadonTorch.cpp:1375-1418) */
enum {
    DD_OP_PROJ = 0,     /* Proj*:                  image -> sinogram (A)          */
    DD_OP_PROJ_T = 1,   /* ProjTrans*:             sinogram -> image (A^T, exact) */
    DD_OP_BPROJ = 2,    /* BackProj*:              sinogram -> image (DD-BP)      */
    DD_OP_BPROJ_T = 3,  /* BackProjTrans*:         image -> sinogram              */
    DD_OP_BPROJ_W = 4,  /* BackProjWeighted*:      FBP-weighted DD-BP             */
    DD_OP_BPROJ_TW = 5  /* BackProjTransWeighted*: its transpose                  */
};

/* 2-D geometry: the 11 entries of projector2d.options (projector.py:113).
 * For fan-arc, det_size and bin_shift are angles (projector.py:110-112). */
typedef struct dd_geom2d {
    int width, height, num_det;
    float pix_x, pix_y, det_size, iso_source, source_detector;
    float pix_xshift, pix_yshift, bin_shift;
} dd_geom2d;

/* 3-D geometry: the 17 entries of projector3d.options (projector.py:286);
 * projectorsp has no z shift (projector.py:460), pass pix_zshift = 0. */
typedef struct dd_geom3d {
    int width, height, depth, num_col, num_row;
    float pix_x, pix_y, pix_z, col_size, row_size, iso_source, source_detector;
    float pix_xshift, pix_yshift, pix_zshift, col_shift, row_shift;
} dd_geom3d;

/* ---- 2-D: argument validation (no device work) ---------------------------
 * The checks every 2-D entry performs before enqueuing anything: returns
 * DD_ERR_INVALID_ARG / DD_ERR_SIZE_OVERFLOW / DD_ERR_UNSUPPORTED or DD_OK.
 * The reference checks only device and contiguity (RadonTorch.cpp:12-14). */
int dd2d_validate(int scan, int op, const dd_geom2d *g, int batch, int num_view);

/* ---- 2-D: generic entry --------------------------------------------------
 * in/out/angles are device pointers; out is fully overwritten.
 * Replaces the 16 2-D radontorch operators, e.g. ProjFanFlatDis2d
 * (RadonTorch.cpp:17-49) for scan=DD_SCAN_FLAT, op=DD_OP_PROJ. */
size_t dd2d_workspace_bytes(int scan, int op, const dd_geom2d *g, int batch, int num_view);
int dd2d_apply(int scan, int op, const dd_geom2d *g, const float *in, float *out,
               const float *angles, int batch, int num_view, void *workspace,
               size_t workspace_bytes, dd_stream_t stream);

/* ---- 2-D: geometry plan reuse ------------------------------------------
 * The per-view / per-line geometry (detector boundary tables and the drifted
 * pixel-boundary pieces) depends only on (scan, geometry, angles).  Building
 * it once and passing it to dd2d_apply_planned saves the set-up kernels in
 * iterative loops (and keeps them out of captured graphs). */
size_t dd2d_plan_bytes(int scan, const dd_geom2d *g, int num_view);
int dd2d_plan(int scan, const dd_geom2d *g, const float *angles, int num_view, void *plan,
              size_t plan_bytes, dd_stream_t stream);
size_t dd2d_apply_workspace_bytes(int scan, int op, const dd_geom2d *g, int batch, int num_view);
int dd2d_apply_planned(int scan, int op, const dd_geom2d *g, const void *plan, const float *in,
                       float *out, int batch, int num_view, void *workspace,
                       size_t workspace_bytes, dd_stream_t stream);

/* ---- 2-D: data-consistency step -------------------------------------------
 * x <- x - eta * A^T (A x - y) for a batch of slices sharing one geometry:
 * the forward writes the residual A x - y into `resid` (B, V, D) directly and
 * the exact adjoint updates x in place.  No counterpart in the reference: the
 * PrideDiff caller builds it from two separate operator calls
 * (model/pridediff.py:56-68).  `plan` from dd2d_plan; workspace size from
 * dd2d_dc_workspace_bytes.  Capturable in a CUDA graph. */
size_t dd2d_dc_workspace_bytes(int scan, const dd_geom2d *g, int batch, int num_view);
int dd2d_dc_step(int scan, const dd_geom2d *g, const void *plan, float *x, const float *y, float *resid,
                 float eta, int batch, int num_view, void *workspace, size_t workspace_bytes,
                 dd_stream_t stream);

/* ---- 2-D: uneven batches in one persistent launch --------------------------
 * No counterpart in the reference, which runs one uniform geometry per call
 * (batch folded into gridDim.x, ParaDisCUDA2d.cu:334-337).  An uneven batch
 * is n instances of one scan type, each with its own geometry, view count and
 * number of slices.  Inputs and outputs are packed instance after instance:
 * images (batch_i, H_i, W_i), sinograms (batch_i, V_i, D_i).  Weighted
 * operators are not batched, and instances whose walked lines are too long
 * for the persistent forward's shared memory (about 3,400 pixels) are refused
 * with DD_ERR_SIZE_OVERFLOW (the single-geometry entry points take them). */
typedef struct dd_instance2d {
    dd_geom2d geom;
    int num_view;
    int batch;        /* slices sharing this geometry */
} dd_instance2d;

/* launch shapes chosen by the autotuner (pridediff_gb300/autotune.py); zero
 * fields take the defaults.  No counterpart in the reference (its launch
 * shape is fixed, BLOCK_DIM 256).  Persistent (uneven-batch) launches: */
typedef struct dd_tune2d {
    int ctas_per_sm;    /* persistent CTAs per SM (0 = as many as fit; capped at that) */
    int lpt_order;      /* items longest-first (1) or in instance order (0) */
    /* single-geometry forward (dd2d_apply_planned_tuned): */
    int fwd_slices;     /* slices per CTA: 4 (default) or 1 */
    int fwd_cluster;    /* CTAs sharing a view's walked lines, a cluster: 2 (default) or 1 */
    /* persistent forward: */
    int items_cluster;  /* CTAs sharing an item's walked lines: 1 (default) or 2 */
    int reserved[3];
} dd_tune2d;

/* dd2d_apply_planned with the single-geometry forward's CTA shape taken from
 * `tune` (fwd_slices, fwd_cluster; NULL = defaults). */
int dd2d_apply_planned_tuned(int scan, int op, const dd_geom2d *g, const void *plan, const float *in,
                             float *out, int batch, int num_view, void *workspace, size_t workspace_bytes,
                             const dd_tune2d *tune, dd_stream_t stream);
/* The forward CTA shape a tune resolves to on this geometry (slices per CTA,
 * cluster size): 4 slices become 2 where their line tables would not fit in
 * shared memory. */
int dd2d_fwd_shape(int scan, const dd_geom2d *g, const dd_tune2d *tune, int *slices, int *cluster);

size_t dd2d_batch_plan_bytes(int scan, const dd_instance2d *inst, int n);
size_t dd2d_batch_workspace_bytes(int scan, const dd_instance2d *inst, int n);
/* Builds every instance's plan and the work lists.  angles[i] is the device
 * pointer of instance i's angles.  Synchronises `stream` (plan time only). */
int dd2d_batch_plan(int scan, const dd_instance2d *inst, int n, const float *const *angles, void *plan,
                    size_t plan_bytes, const dd_tune2d *tune, dd_stream_t stream);
int dd2d_batch_apply(int scan, int op, const dd_instance2d *inst, int n, const void *plan, const float *in,
                     float *out, void *workspace, size_t workspace_bytes, const dd_tune2d *tune,
                     dd_stream_t stream);
/* x <- x - eta * A^T (A x - y) over all instances (packed x and y). */
int dd2d_batch_dc_step(int scan, const dd_instance2d *inst, int n, const void *plan, float *x, const float *y,
                       float eta, void *workspace, size_t workspace_bytes, const dd_tune2d *tune,
                       dd_stream_t stream);
/* Device status word of the last batched call (DD_OK or DD_ERR_TIMEOUT);
 * synchronous. */
int dd2d_batch_status(int scan, const dd_instance2d *inst, int n, const void *workspace, int *status);

/* ---- device-side timeouts -------------------------------------------------
 * No counterpart in the reference (it checks no CUDA error at all,
 * RadonTorch.cpp:12-14 is its only validation).  Every wait of a kernel on an
 * asynchronous copy is bounded; a wait that gives up makes the kernel skip
 * the rest of its work, let its copies in flight land, record DD_ERR_TIMEOUT
 * and return, so the context stays usable.  The record is kept in the
 * status word of the call's workspace, read synchronously by: */
/* dd2d_apply / dd_<Name>Dis2d on `workspace` (same arguments as the call) */
int dd2d_status(int scan, int op, const dd_geom2d *g, int batch, int num_view, const void *workspace,
                int *status);
/* dd2d_apply_planned / dd2d_dc_step on `workspace` (the apply workspace) */
int dd2d_planned_status(int op, const dd_geom2d *g, int batch, int num_view, const void *workspace,
                        int *status);
/* and, without any synchronisation, in one word of pinned, device-mapped
 * host memory registered here (per device: call once with each device
 * current; NULL unregisters).  Kernels write DD_ERR_TIMEOUT into it with a
 * system-scope atomic; the caller reads and clears it. */
int dd_set_status_sink(int *pinned_host_word);

/* ---- 2-D: named entries, one per radontorch function --------------------
 * Same arguments as dd2d_apply without scan/op.  Each replaces the pybind
 * function of the same name (RadonTorch.cpp:1376-1393). */
#define DD_NAMED2D(name)                                                            \
    int dd_##name(const dd_geom2d *g, const float *in, float *out, const float *angles, \
                  int batch, int num_view, void *workspace, size_t workspace_bytes,      \
                  dd_stream_t stream)
DD_NAMED2D(ProjFanFlatDis2d);               /* RadonTorch.cpp:17   */
DD_NAMED2D(ProjTransFanFlatDis2d);          /* RadonTorch.cpp:52   */
DD_NAMED2D(BackProjFanFlatDis2d);           /* RadonTorch.cpp:86   */
DD_NAMED2D(BackProjTransFanFlatDis2d);      /* RadonTorch.cpp:120  */
DD_NAMED2D(BackProjWeightedFanFlatDis2d);   /* RadonTorch.cpp:154  */
DD_NAMED2D(BackProjTransWeightedFanFlatDis2d); /* RadonTorch.cpp:188 */
DD_NAMED2D(ProjFanArcDis2d);                /* RadonTorch.cpp:225  */
DD_NAMED2D(ProjTransFanArcDis2d);           /* RadonTorch.cpp:260  */
DD_NAMED2D(BackProjFanArcDis2d);            /* RadonTorch.cpp:294  */
DD_NAMED2D(BackProjTransFanArcDis2d);       /* RadonTorch.cpp:328  */
DD_NAMED2D(BackProjWeightedFanArcDis2d);    /* RadonTorch.cpp:362  */
DD_NAMED2D(BackProjTransWeightedFanArcDis2d); /* RadonTorch.cpp:396 */
DD_NAMED2D(ProjParaDis2d);                  /* RadonTorch.cpp:433  */
DD_NAMED2D(ProjTransParaDis2d);             /* RadonTorch.cpp:468  */
DD_NAMED2D(BackProjParaDis2d);              /* RadonTorch.cpp:502  */
DD_NAMED2D(BackProjTransParaDis2d);         /* RadonTorch.cpp:536  */
#undef DD_NAMED2D

/* ---- 2-D: system matrix ----------------------------------------------------
 * Replaces GetSysMatrixPara2d / GetSysMatrixFanFlat2d / GetSysMatrixFanArc2d
 * (RadonTorch.cpp:1270-1372): the COO matrix (V*D x H*W) with one entry per
 * step of the DD merge walk, in the reference's order (view, walked line,
 * step).  The reference builds it on the CPU; here it is built on the device
 * in two passes over a plan from dd2d_plan:
 *   1. dd2d_sysmatrix_count writes the entries of each (view, walked line)
 *      into counts[dd2d_sysmatrix_lines()], index view * max(H, W) + line;
 *   2. the caller takes the exclusive prefix sum of counts as offsets and
 *      allocates nnz = sum(counts) rows / cols (int64) and vals (FP32);
 *   3. dd2d_sysmatrix_fill writes the entries. */
size_t dd2d_sysmatrix_lines(const dd_geom2d *g, int num_view);
int dd2d_sysmatrix_count(int scan, const dd_geom2d *g, const void *plan, int num_view, long long *counts,
                         dd_stream_t stream);
int dd2d_sysmatrix_fill(int scan, const dd_geom2d *g, const void *plan, int num_view, const long long *offsets,
                        long long *rows, long long *cols, float *vals, dd_stream_t stream);

/* ---- FBP filtering ---------------------------------------------------------
 * Replaces `nn.functional.conv2d(sino * weight, filter, padding=(0, D - 1))`
 * (conv3d for the 3-D geometries) in deeprecon's filtered_backprojection
 * (deeprecon/torch/projector/projector.py:192-213, 368-390, 554-563): for
 * `rows` detector rows of num_det bins,
 *   out[i][k] = sum_n taps[n - k + num_det - 1] * (weight[i % wrows][n] * in[i][n]),
 * taps holding 2 num_det - 1 entries (filter.py:8-30 builds them).  weight
 * may be NULL (unit weight).  Device pointers; out must not alias in. */
int dd_fbp_filter(const float *in, float *out, const float *weight, int wrows, const float *taps,
                  long long rows, int num_det, dd_stream_t stream);

/* ---- 3-D: cone-flat, cone-arc, spiral --------------------------------------
 * Same conventions as 2-D.  source_pos is the spiral source table (4, V) on
 * the device (RadonTorch.cpp:1040-1043); pass NULL for the cone geometries.
 * The reference has no CPU path for 3-D (RadonTorch.cpp:604). */
int dd3d_validate(int scan, int op, const dd_geom3d *g, int batch, int num_view);
size_t dd3d_workspace_bytes(int scan, int op, const dd_geom3d *g, int batch, int num_view);
int dd3d_apply(int scan, int op, const dd_geom3d *g, const float *in, float *out, const float *angles,
               const float *source_pos, int batch, int num_view, void *workspace, size_t workspace_bytes,
               dd_stream_t stream);
/* plan reuse: per-view column / row tables and the per-(view, line, 256-column
 * block) drift records (the reference restarts its FP32 walk per block,
 * ConeFlatDisCUDA3d.cu:53-56) */
size_t dd3d_plan_bytes(int scan, const dd_geom3d *g, int num_view);
int dd3d_plan(int scan, const dd_geom3d *g, const float *angles, const float *source_pos, int num_view,
              void *plan, size_t plan_bytes, dd_stream_t stream);
size_t dd3d_apply_workspace_bytes(int scan, int op, const dd_geom3d *g, int batch, int num_view);
int dd3d_apply_planned(int scan, int op, const dd_geom3d *g, const void *plan, const float *in, float *out,
                       int batch, int num_view, void *workspace, size_t workspace_bytes, dd_stream_t stream);
/* x <- x - eta * A^T (A x - y) (no counterpart in the reference; the PrideDiff
 * caller composes two operator calls, model/pridediff.py:56-68) */
size_t dd3d_dc_workspace_bytes(int scan, const dd_geom3d *g, int batch, int num_view);
int dd3d_dc_step(int scan, const dd_geom3d *g, const void *plan, float *x, const float *y, float *resid,
                 float eta, int batch, int num_view, void *workspace, size_t workspace_bytes, dd_stream_t stream);
/* Status word (DD_OK or DD_ERR_TIMEOUT) of the last dd3d_apply on `workspace`
 * (same arguments as the call), or of the last dd3d_apply_planned on its
 * apply workspace; synchronous (see "device-side timeouts" above). */
int dd3d_status(int scan, int op, const dd_geom3d *g, int batch, int num_view, const void *workspace,
                int *status);
int dd3d_planned_status(int op, const dd_geom3d *g, int batch, int num_view, const void *workspace, int *status);

/* named entries, one per 3-D radontorch function (RadonTorch.cpp:1395-1414) */
#define DD_NAMED3D(name)                                                                          \
    int dd_##name(const dd_geom3d *g, const float *in, float *out, const float *angles,           \
                  const float *source_pos, int batch, int num_view, void *workspace,              \
                  size_t workspace_bytes, dd_stream_t stream)
DD_NAMED3D(ProjConeFlatDis3d);                  /* RadonTorch.cpp:572  */
DD_NAMED3D(ProjTransConeFlatDis3d);             /* RadonTorch.cpp:609  */
DD_NAMED3D(BackProjConeFlatDis3d);              /* RadonTorch.cpp:646  */
DD_NAMED3D(BackProjTransConeFlatDis3d);         /* RadonTorch.cpp:683  */
DD_NAMED3D(BackProjWeightedConeFlatDis3d);      /* RadonTorch.cpp:720  */
DD_NAMED3D(BackProjTransWeightedConeFlatDis3d); /* RadonTorch.cpp:757  */
DD_NAMED3D(ProjConeArcDis3d);                   /* RadonTorch.cpp:795  */
DD_NAMED3D(ProjTransConeArcDis3d);              /* RadonTorch.cpp:832  */
DD_NAMED3D(BackProjConeArcDis3d);               /* RadonTorch.cpp:869  */
DD_NAMED3D(BackProjTransConeArcDis3d);          /* RadonTorch.cpp:906  */
DD_NAMED3D(BackProjWeightedConeArcDis3d);       /* RadonTorch.cpp:943  */
DD_NAMED3D(BackProjTransWeightedConeArcDis3d);  /* RadonTorch.cpp:980  */
DD_NAMED3D(ProjSpiralDis3d);                    /* RadonTorch.cpp:1018 */
DD_NAMED3D(ProjTransSpiralDis3d);               /* RadonTorch.cpp:1060 */
DD_NAMED3D(BackProjSpiralDis3d);                /* RadonTorch.cpp:1102 */
DD_NAMED3D(BackProjTransSpiralDis3d);           /* RadonTorch.cpp:1144 */
DD_NAMED3D(BackProjWeightedSpiralDis3d);        /* RadonTorch.cpp:1186 */
DD_NAMED3D(BackProjTransWeightedSpiralDis3d);   /* RadonTorch.cpp:1228 */
#undef DD_NAMED3D

/* ---- 2-D: forward projection without any caller workspace ----------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (a plugin whose host framework owns all device memory, a real-time
 * loop that may not touch the allocator): same computation as
 * dd_ProjFanFlatDis2d, with its scratch taken from a 32 MiB buffer that is
 * part of the library (kept on every GPU that loads the library until the
 * process exits).  Problems needing more scratch than that
 * (dd2d_workspace_bytes) are refused with DD_ERR_WORKSPACE.  The first call
 * on a device resolves the buffer's address; make it before any stream
 * capture.  Calls share the buffer: calls that overlap on the GPU race. */
int dd_ProjFanFlatDis2d_noalloc(const dd_geom2d *g, const float *in, float *out, const float *angles,
                                int batch, int num_view, dd_stream_t stream);
/* Status word (DD_OK or DD_ERR_TIMEOUT) of the last no-allocation call on the
 * current device, read from the library's buffer; synchronous.  The buffer's
 * address is resolved once per device and kept: do not call these after
 * cudaDeviceReset on that device. */
int dd_noalloc_status(int *status);

/* ---- diagnostics ----------------------------------------------------------
 * No counterpart in the reference (it has no instrumentation).  Kernel kinds
 * for dd_profile_read: */
enum { DD_KERNEL_FORWARD = 0, DD_KERNEL_ADJOINT = 1, DD_KERNEL_TABLES = 2, DD_KERNEL_PLAN = 3, DD_KERNEL_FILTER = 4 };
/* Number of kernels this library has launched in the process. */
unsigned long long dd_launch_count(void);
/* Record CUDA events around every subsequent launch (and reset the records);
 * must not be enabled while a stream is being captured. */
int dd_profile_enable(int on);
/* Sum of the recorded durations (ms) and launch count of one kernel kind;
 * synchronises on the recorded events. */
int dd_profile_read(int kind, double *total_ms, int *count);
const char *dd_status_string(int status);
/* Library version and build target, e.g. "pridediff_dd 0.2 sm_103a"; part of
 * the autotuner's cache key, so choices recorded by another version are not reused. */
const char *dd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PRIDEDIFF_DD_H */
