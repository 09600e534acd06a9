// Batched 2-D DD projection over uneven instances in one persistent launch.
//
// An uneven batch is a list of instances, each with its own image size,
// view count, detector count and number of slices (one scan type per batch).
// The reference has no batching beyond folding the batch into gridDim.x with
// one uniform geometry per call (ParaDisCUDA2d.cu:334-337); here every
// instance's geometry plan lives in one plan buffer, the work of all
// instances is cut into items (forward: one view x a group of slices;
// adjoint: one 32x32 tile x a group of slices), and a persistent grid of
// `ctas_per_sm` CTAs per SM pulls items from a device counter in
// longest-first order.  The item bodies are the single-geometry ones
// (dd2d_kernels.cuh), so results are identical to per-instance calls.
//
// The data-consistency step x <- x - eta * A^T (A x - y) is four launches:
// image tables, forward items writing the residual A x - y directly, detector
// tables of the residual, adjoint items updating x in place.  No host syncs,
// no allocations: the step is capturable in a CUDA graph.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "dd2d_kernels.cuh"
#include "dd_trace.h"

namespace dd2 {

struct BatchInst {
    dd_geom2d g;
    int V, batch, nl, pad;
    long long plan_off;            // bytes: instance plan inside the batch plan
    long long img_off, sino_off;   // elements: packed images / sinograms
    long long tabx_off, taby_off;  // float2: forward tables in the workspace
    long long dtab_off;            // float2: adjoint tables in the workspace
    long long views, ang, dp, bcoef, lines, dlines, amap, trange;   // PlanLayout offsets
};

struct BatchLayout {
    size_t desc, fitems, aitems, plans, total;        // plan buffer
    size_t w_tabs, w_dtab, w_resid, w_counter, w_status, w_total;   // workspace
    int nfwd, nadj, Dmax, rsmax;
    int fi;   // slices per forward item (fwd_item_slices)
    std::vector<BatchInst> inst;
};

// Slices per persistent forward item: 2 where no instance has more than 2
// slices (after instances with one geometry are merged, the usual uneven
// batch), so that the forward kernel holds half the line tables and runs 6
// CTAs per SM instead of 5 (24 uneven instances: 6.51 -> 6.16 ms); kBI
// otherwise, where 4 slices share each locate.
static int fwd_item_slices(const dd_instance2d *in, int n) {
    int mb = 0;
    for (int i = 0; i < n; i++) mb = std::max(mb, in[i].batch);
    return mb <= 2 ? 2 : kBI;
}

static BatchLayout batch_layout(int scan, const dd_instance2d *in, int n, int bi) {
    BatchLayout L;
    L.inst.resize(n);
    L.fi = fwd_item_slices(in, n);
    long long img = 0, sino = 0, tabs = 0, dtab = 0;
    size_t plans = 0;
    L.nfwd = L.nadj = 0;
    L.Dmax = 1;
    L.rsmax = 2;
    for (int i = 0; i < n; i++) {
        BatchInst &d = L.inst[i];
        memset(&d, 0, sizeof(d));
        d.g = in[i].geom;
        d.V = in[i].num_view;
        d.batch = in[i].batch;
        const PlanLayout P = plan_layout(scan, &d.g, d.V);
        d.nl = P.nl;
        d.plan_off = (long long)plans;
        plans = align_up(plans + P.total, 256);
        d.views = (long long)P.views;
        d.ang = (long long)P.ang;
        d.dp = (long long)P.dp;
        d.bcoef = (long long)P.bcoef;
        d.lines = (long long)P.lines;
        d.dlines = (long long)P.dlines;
        d.amap = (long long)P.amap;
        d.trange = (long long)P.trange;
        const int W = d.g.width, H = d.g.height, D = d.g.num_det;
        d.img_off = img;
        img += (long long)d.batch * H * W;
        d.sino_off = sino;
        sino += (long long)d.batch * d.V * D;
        d.tabx_off = tabs;
        tabs += (long long)d.batch * H * rs_entries(W);
        d.taby_off = tabs;
        tabs += (long long)d.batch * W * rs_entries(H);
        tabs = (tabs + 1) & ~1LL;
        d.dtab_off = dtab;
        dtab += ((long long)d.batch * d.V * rs_entries(D) + 1) & ~1LL;
        const int groups = (d.batch + bi - 1) / bi;
        L.nfwd += d.V * ((d.batch + L.fi - 1) / L.fi);
        L.nadj += ((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile) * groups;
        L.Dmax = std::max(L.Dmax, D);
        L.rsmax = std::max(L.rsmax, rs_entries(std::max(W, H)));
    }
    size_t o = 0;
    L.desc = o; o = align_up(o + sizeof(BatchInst) * (size_t)n, 256);
    L.fitems = o; o = align_up(o + sizeof(int4) * (size_t)L.nfwd, 256);
    L.aitems = o; o = align_up(o + sizeof(int4) * (size_t)L.nadj, 256);
    L.plans = o; o = align_up(o + plans, 256);
    L.total = o;
    size_t w = 0;
    L.w_tabs = w; w = align_up(w + sizeof(float2) * (size_t)tabs, 256);
    L.w_dtab = w; w = align_up(w + sizeof(float2) * (size_t)dtab, 256);
    L.w_resid = w; w = align_up(w + sizeof(float) * (size_t)sino, 256);
    L.w_counter = w; w = align_up(w + 2 * sizeof(int), 256);
    L.w_status = w; w = align_up(w + sizeof(int), 256);
    L.w_total = w;
    return L;
}

// ---------------------------------------------------------------------------
// Batched prefix tables (one launch each; blockIdx.y = instance)
// ---------------------------------------------------------------------------
__global__ void k_tab_rows_b(const BatchInst *__restrict__ desc, const float *__restrict__ img,
                             float2 *__restrict__ tabs) {
    const BatchInst &d = desc[blockIdx.y];
    const int W = d.g.width, H = d.g.height;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= d.batch * H) return;
    const float *row = img + d.img_off + (size_t)warp * W;
    warp_prefix_table(W, tabs + d.tabx_off + (size_t)warp * rs_entries(W), lane, [&](int j, float *x, float *w) {
        *x = row[j];
        *w = 1.0f;
    });
}

// Column tables as the single-geometry k_tab_cols builds them: a block takes
// 32 of an instance's (image, column) lines, its 8 warps a chunk of rows each.
__global__ void __launch_bounds__(256) k_tab_cols_b(const BatchInst *__restrict__ desc,
                                                    const float *__restrict__ img, float2 *__restrict__ tabs) {
    constexpr int kChunks = 8;
    const BatchInst &d = desc[blockIdx.y];
    const int W = d.g.width, H = d.g.height;
    const int c = threadIdx.x & 31, k = threadIdx.x >> 5;
    const int idx = blockIdx.x * 32 + c;
    const bool ok = idx < d.batch * W;
    const int b = ok ? idx / W : 0, col = ok ? idx - b * W : 0;
    const int per = (H + kChunks - 1) / kChunks;
    const int i0 = min(H, k * per), i1 = min(H, i0 + per);
    const float *__restrict__ im = img + d.img_off + (size_t)b * H * W + col;
    __shared__ float tot_hi[kChunks][32], tot_lo[kChunks][32];
    DdF run = {0.0f, 0.0f};
    if (ok)
        for (int i = i0; i < i1; i++) run = df_add(run, DdF{__ldg(im + (size_t)(H - 1 - i) * W), 0.0f});
    tot_hi[k][c] = run.hi;
    tot_lo[k][c] = run.lo;
    __syncthreads();
    if (!ok) return;
    run = {0.0f, 0.0f};
    for (int q = 0; q < k; q++) run = df_add(run, DdF{tot_hi[q][c], tot_lo[q][c]});
    float2 *__restrict__ t = tabs + d.taby_off + (size_t)idx * rs_entries(H);
    for (int i = i0; i < i1; i++) {
        const float x = __ldg(im + (size_t)(H - 1 - i) * W);
        t[i] = make_float2(run.hi, x);
        run = df_add(run, DdF{x, 0.0f});
    }
    if (i0 < H && i1 == H) t[H] = make_float2(run.hi, 0.0f);
}

__global__ void k_dettab_b(int geom, int mode, const BatchInst *__restrict__ desc,
                           const char *__restrict__ plan, size_t plans_off,
                           const float *__restrict__ sino, float2 *__restrict__ dtabs) {
    const BatchInst &d = desc[blockIdx.y];
    const int V = d.V, D = d.g.num_det;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= d.batch * V) return;
    const int b = warp / V, v = warp - b * V;
    const char *pb = plan + plans_off + d.plan_off;
    const DdView2 vw = reinterpret_cast<const DdView2 *>(pb + d.views)[v];
    const float *dpv = reinterpret_cast<const float *>(pb + d.dp) + (size_t)v * (D + 1);
    const float *bc = reinterpret_cast<const float *>(pb + d.bcoef) + (size_t)v * (D + 1);
    const float *s = sino + d.sino_off + ((size_t)b * V + v) * D;
    float2 *t = dtabs + d.dtab_off + (size_t)warp * rs_entries(D);
    const float pc = vw.xb ? d.g.pix_y / d.g.det_size : d.g.pix_x / d.g.det_size;
    warp_prefix_table(D, t, lane, [&](int k, float *g, float *w) {
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

// ---------------------------------------------------------------------------
// Persistent item kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ int next_item(int *counter) {
    __shared__ int s_item;
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    return s_item;
}

// The forward's clusters: rank 0 takes the next item, the other ranks read its
// index from rank 0's shared memory.  The second barrier keeps rank 0 (and
// its s_item) in place until every rank has read it: past the last item rank
// 0 exits, and a CTA's shared memory must not be read after it has exited.
__device__ __forceinline__ int next_item_cluster(int *counter) {
    __shared__ int s_item;
    cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
    if (cluster.block_rank() == 0 && threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    cluster.sync();
    const int i = *cluster.map_shared_rank(&s_item, 0);
    cluster.sync();
    return i;
}

// Resident CTAs per SM the persistent forward is compiled for: items of 4
// slices, 48 registers per thread up to 4 passes (on 24 uneven one-slice
// instances 5 CTAs per SM ran the forward in 8.13 ms, 6 in 8.20 ms); items
// of 2 slices, 40 registers and 6 CTAs.
__host__ __device__ constexpr int fwd_items_min_ctas(int npass, int bi) {
    return npass <= 4 ? (bi <= 2 ? 6 : 5) : 3;
}

// CTAs per persistent-forward cluster.  Batches of many short items leave
// little tail to split: on 24 uneven one-slice instances, clusters of 2 (an
// item's lines shared as in the single-geometry forward) took 9.00 ms, single
// CTAs 8.20 ms.  A single CTA sums a view's lines in one sequence, the
// single-geometry forward's cluster as two interleaved halves, so the two
// projections of an instance agree to FP32 rounding, not bit for bit
// (walking the lines in the cluster's order cost 8.73 vs 8.13 ms).
// The cluster size is a tuning choice (dd_tune2d.items_cluster): 1 unless the
// autotuner finds 2 faster for the batch at hand.
constexpr int kFwdItemsCluster = 1;

template <int GEOM, int NPASS, int CL, int BI>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(kThreads, fwd_items_min_ctas(NPASS, BI))
k_fwd_items(int op, const BatchInst *__restrict__ desc, const int4 *__restrict__ items, int nitems,
            const char *__restrict__ plan, size_t plans_off, const float2 *__restrict__ tabs,
            float *__restrict__ out, const float *__restrict__ sub, int Dmax, int rsmax,
            int *__restrict__ counter, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const FwdSmem L = fwd_smem(GEOM, Dmax, rsmax, BI, CL);
    init_bars(reinterpret_cast<uint64_t *>(smem + L.bar));
    // the item and its geometry live in shared memory: read where used, they
    // hold no registers across the line loop (the plain forward reads them
    // from kernel parameters)
    __shared__ FwdItem s_it;
    __shared__ dd_geom2d s_g;
    DdPhases ph;
    for (;;) {
        int i;
        if constexpr (CL > 1) i = next_item_cluster(counter);
        else i = next_item(counter);
        if (i >= nitems) break;
        if (threadIdx.x == 0) {
            const int4 w = items[i];
            const BatchInst &d = desc[w.x];
            const char *pb = plan + plans_off + d.plan_off;
            FwdItem it;
            it.v = w.y;
            it.b0 = w.z;
            it.nb = w.w;
            it.V = d.V;
            it.nl = d.nl;
            it.views = reinterpret_cast<const DdView2 *>(pb + d.views);
            it.dp = reinterpret_cast<const float *>(pb + d.dp);
            it.bcoef = reinterpret_cast<const float *>(pb + d.bcoef);
            it.lines = reinterpret_cast<const DdLine *>(pb + d.lines);
            it.dlines = reinterpret_cast<const DdLine *>(pb + d.dlines);
            it.tabx = tabs + d.tabx_off;
            it.taby = tabs + d.taby_off;
            it.out = out + d.sino_off;
            it.sub = sub ? sub + d.sino_off : nullptr;
            s_it = it;
            s_g = d.g;
        }
        __syncthreads();   // every thread passed the cluster barrier above before s_it changes
        if (!fwd_view<GEOM, 0, NPASS, BI, kWarps, CL>(s_g, op, s_it, smem, Dmax, rsmax, ph)) {
            if (threadIdx.x == 0) dd_report_timeout(status);
            break;
        }
    }
}

// Fan beams: held to the plain adjoint's 4 CTAs per SM (64 registers per
// thread); parallel beams (two sets of accumulators): 3.  The item and its
// geometry live in shared memory, as in the forward.
template <int GEOM, int OPK>
__global__ void __launch_bounds__(kThreads, GEOM == DD_GEOM_PARA ? 3 : 4)
k_adj_items(const BatchInst *__restrict__ desc, const int4 *__restrict__ items, int nitems,
            const char *__restrict__ plan, size_t plans_off, const float2 *__restrict__ dtabs,
            float *__restrict__ out, const float *__restrict__ base, float scale,
            int *__restrict__ counter, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const AdjSmem SL = adj_smem(GEOM);
    init_bars(reinterpret_cast<uint64_t *>(smem + SL.bar), GEOM == DD_GEOM_PARA ? 2 : kAdjBufs);
    __shared__ AdjItem s_it;
    __shared__ dd_geom2d s_g;
    DdPhases ph;
    for (;;) {
        const int i = next_item(counter + 1);   // its barriers also order s_it's reuse
        if (i >= nitems) break;
        if (threadIdx.x == 0) {
            const int4 w = items[i];
            const BatchInst &d = desc[w.x];
            const char *pb = plan + plans_off + d.plan_off;
            AdjItem it;
            it.c0 = (w.y & 0xFFFF) * kTile;
            it.r0 = (w.y >> 16) * kTile;
            it.b0 = w.z;
            it.nb = w.w;
            it.V = d.V;
            it.nl = d.nl;
            it.angles = reinterpret_cast<const float *>(pb + d.ang);
            it.views = reinterpret_cast<const DdView2 *>(pb + d.views);
            it.dp = reinterpret_cast<const float *>(pb + d.dp);
            it.lines = reinterpret_cast<const DdLine *>(pb + d.lines);
            it.dlines = reinterpret_cast<const DdLine *>(pb + d.dlines);
            it.amap = reinterpret_cast<const unsigned char *>(pb + d.amap);
            it.trange = reinterpret_cast<const int2 *>(pb + d.trange);
            it.dtab = dtabs + d.dtab_off;
            it.out = out + d.img_off;
            it.base = base ? base + d.img_off : nullptr;
            it.scale = scale;
            s_it = it;
            s_g = d.g;
        }
        __syncthreads();
        bool ok;
        if constexpr (GEOM == DD_GEOM_PARA) ok = adj_tile<GEOM, OPK>(s_g, s_it, smem, ph);
        else ok = adj_tile_map<GEOM, OPK>(s_g, s_it, smem, ph);
        if (!ok) {
            if (threadIdx.x == 0) dd_report_timeout(status);
            break;
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 1;
    }
    return n;
}

static int validate_batch(int scan, int op, const dd_instance2d *inst, int n) {
    if (!inst || n <= 0 || n > 65535) return DD_ERR_INVALID_ARG;
    if (op == DD_OP_BPROJ_W || op == DD_OP_BPROJ_TW) return DD_ERR_UNSUPPORTED;
    for (int i = 0; i < n; i++) {
        const int st = validate(scan, op, &inst[i].geom, inst[i].batch, inst[i].num_view);
        if (st != DD_OK) return st;
        if ((inst[i].geom.width + kTile - 1) / kTile > 0xFFFF) return DD_ERR_SIZE_OVERFLOW;
        // the persistent forward stages 4 images' line tables per CTA
        const dd_geom2d &g = inst[i].geom;
        if (fwd_smem(geom_of(scan), g.num_det, rs_entries(std::max(g.width, g.height)), kBI,
                     kFwdItemsCluster).total > max_smem_optin())
            return DD_ERR_SIZE_OVERFLOW;
    }
    return DD_OK;
}

// Persistent grid: CTAs per SM as the tuning asks, at most as many as fit
// (`fit`, from the kernel's registers and shared memory); 0 = as many as fit.
static int grid_of(const dd_tune2d *t, int nitems, int fit) {
    int per = (t && t->ctas_per_sm > 0) ? t->ctas_per_sm : fit;
    if (per > fit) per = fit;
    if (per < 1) per = 1;
    return std::max(1, std::min(nitems, per * sm_count()));
}

template <typename K>
static int resident_ctas(K kern, int smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kThreads, (size_t)smem) != cudaSuccess || n < 1) n = 1;
    return n;
}

// Persistent grid of a clustered kernel (clusters of `cl` CTAs): grid_of's CTA
// count rounded down to whole clusters, at most the clusters that can be
// resident at once.
template <typename K>
static int cluster_grid_of(const dd_tune2d *t, int nitems, K kern, int smem, int cl) {
    const int ctas = grid_of(t, nitems * cl, resident_ctas(kern, smem));
    int clusters = std::max(1, std::min(nitems, ctas / cl));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusters * cl);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = (size_t)smem;
    int maxc = 0;
    if (cudaOccupancyMaxActiveClusters(&maxc, (void *)kern, &cfg) == cudaSuccess && maxc > 0)
        clusters = std::min(clusters, maxc);
    else
        (void)cudaGetLastError();
    return clusters * cl;
}

template <int GEOM, int CL, int BI>
static auto fwd_items_kernel(int Dmax) {
    auto kern = k_fwd_items<GEOM, 8, CL, BI>;
    switch (npass_class(Dmax)) {
    case 1: kern = k_fwd_items<GEOM, 1, CL, BI>; break;
    case 2: kern = k_fwd_items<GEOM, 2, CL, BI>; break;
    case 3: kern = k_fwd_items<GEOM, 3, CL, BI>; break;
    case 4: kern = k_fwd_items<GEOM, 4, CL, BI>; break;
    default: break;
    }
    return kern;
}

template <int GEOM>
static int launch_fwd_items(int op, const BatchLayout &L, const char *planb, const float2 *tabs,
                            float *out, const float *sub, int *counter, int *status, const dd_tune2d *tune,
                            cudaStream_t st) {
    int cl = (tune && tune->items_cluster == 2) ? 2 : kFwdItemsCluster;
    if (cl == 2 && fwd_smem(GEOM, L.Dmax, L.rsmax, L.fi, 2).total > max_smem_optin()) cl = 1;
    const FwdSmem S = fwd_smem(GEOM, L.Dmax, L.rsmax, L.fi, cl);
    auto kern = (L.fi == 2)
        ? ((cl == 2) ? fwd_items_kernel<GEOM, 2, 2>(L.Dmax) : fwd_items_kernel<GEOM, 1, 2>(L.Dmax))
        : ((cl == 2) ? fwd_items_kernel<GEOM, 2, kBI>(L.Dmax) : fwd_items_kernel<GEOM, 1, kBI>(L.Dmax));
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S.total) != cudaSuccess)
        return DD_ERR_LAUNCH;
    const int grid = cluster_grid_of(tune, L.nfwd, kern, S.total, cl);
    ProfRec *pr = prof_begin(DD_KERNEL_FORWARD, st);
    kern<<<grid, kThreads, S.total, st>>>(op, (const BatchInst *)(planb + L.desc),
                                          (const int4 *)(planb + L.fitems), L.nfwd, planb, L.plans, tabs,
                                          out, sub, L.Dmax, L.rsmax, counter, status);
    prof_end(pr, st);
    count_launches(1);
    return launch_status();
}

template <int GEOM>
static int launch_adj_items(int op, const BatchLayout &L, const char *planb, const float2 *dtabs,
                            float *out, const float *base, float scale, int *counter, int *status,
                            const dd_tune2d *tune, cudaStream_t st) {
    const AdjSmem S = adj_smem(GEOM);
    auto kern = (op == DD_OP_PROJ_T) ? k_adj_items<GEOM, 0> : k_adj_items<GEOM, 1>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S.total) != cudaSuccess)
        return DD_ERR_LAUNCH;
    const int grid = grid_of(tune, L.nadj, resident_ctas(kern, S.total));
    ProfRec *pr = prof_begin(DD_KERNEL_ADJOINT, st);
    kern<<<grid, kThreads, S.total, st>>>((const BatchInst *)(planb + L.desc),
                                          (const int4 *)(planb + L.aitems), L.nadj, planb, L.plans, dtabs,
                                          out, base, scale, counter, status);
    prof_end(pr, st);
    count_launches(1);
    return launch_status();
}

// forward of all instances: out = A in (- sub)
static int batch_forward(int scan, int op, const BatchLayout &L, const char *planb, const float *in,
                         float *out, const float *sub, char *wb, const dd_tune2d *tune, cudaStream_t st) {
    const int geom = geom_of(scan);
    float2 *tabs = (float2 *)(wb + L.w_tabs);
    int *counter = (int *)(wb + L.w_counter);
    int *status = (int *)(wb + L.w_status);
    const BatchInst *desc = (const BatchInst *)(planb + L.desc);
    int maxrows = 1, maxcols = 1;
    for (const BatchInst &d : L.inst) {
        maxrows = std::max(maxrows, d.batch * d.g.height);
        maxcols = std::max(maxcols, d.batch * d.g.width);
    }
    const int n = (int)L.inst.size();
    ProfRec *pr = prof_begin(DD_KERNEL_TABLES, st);
    k_tab_rows_b<<<dim3((maxrows * 32 + 255) / 256, n), 256, 0, st>>>(desc, in, tabs);
    k_tab_cols_b<<<dim3((maxcols + 31) / 32, n), 256, 0, st>>>(desc, in, tabs);
    prof_end(pr, st);
    count_launches(2);
    if (cudaMemsetAsync(counter, 0, 2 * sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    if (geom == DD_GEOM_PARA) return launch_fwd_items<DD_GEOM_PARA>(op, L, planb, tabs, out, sub, counter, status, tune, st);
    if (geom == DD_GEOM_FLAT) return launch_fwd_items<DD_GEOM_FLAT>(op, L, planb, tabs, out, sub, counter, status, tune, st);
    return launch_fwd_items<DD_GEOM_ARC>(op, L, planb, tabs, out, sub, counter, status, tune, st);
}

// adjoint of all instances: out = base + scale * (A^T in)   (base may be null)
static int batch_adjoint(int scan, int op, const BatchLayout &L, const char *planb, const float *in,
                         float *out, const float *base, float scale, char *wb, const dd_tune2d *tune,
                         cudaStream_t st) {
    const int geom = geom_of(scan);
    float2 *dtabs = (float2 *)(wb + L.w_dtab);
    int *counter = (int *)(wb + L.w_counter);
    int *status = (int *)(wb + L.w_status);
    const BatchInst *desc = (const BatchInst *)(planb + L.desc);
    int maxw = 1;
    for (const BatchInst &d : L.inst) maxw = std::max(maxw, d.batch * d.V);
    const int n = (int)L.inst.size();
    ProfRec *pr = prof_begin(DD_KERNEL_TABLES, st);
    k_dettab_b<<<dim3((maxw * 32 + 255) / 256, n), 256, 0, st>>>(geom, op == DD_OP_PROJ_T ? 0 : 1, desc,
                                                                  planb, L.plans, in, dtabs);
    prof_end(pr, st);
    count_launches(1);
    if (cudaMemsetAsync(counter, 0, 2 * sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    if (geom == DD_GEOM_PARA) return launch_adj_items<DD_GEOM_PARA>(op, L, planb, dtabs, out, base, scale, counter, status, tune, st);
    if (geom == DD_GEOM_FLAT) return launch_adj_items<DD_GEOM_FLAT>(op, L, planb, dtabs, out, base, scale, counter, status, tune, st);
    return launch_adj_items<DD_GEOM_ARC>(op, L, planb, dtabs, out, base, scale, counter, status, tune, st);
}

}  // namespace dd2

using namespace dd2;

extern "C" size_t dd2d_batch_plan_bytes(int scan, const dd_instance2d *inst, int n) {
    if (validate_batch(scan, DD_OP_PROJ, inst, n) != DD_OK) return 0;
    return batch_layout(scan, inst, n, kBI).total;
}

extern "C" size_t dd2d_batch_workspace_bytes(int scan, const dd_instance2d *inst, int n) {
    if (validate_batch(scan, DD_OP_PROJ, inst, n) != DD_OK) return 0;
    return batch_layout(scan, inst, n, kBI).w_total;
}

extern "C" int dd2d_batch_plan(int scan, const dd_instance2d *inst, int n, const float *const *angles,
                               void *planp, size_t plan_bytes, const dd_tune2d *tune, dd_stream_t stream) {
    ddtrace::Range tr("dd2d_batch_plan", scan, -1, false);
    const int vs = validate_batch(scan, DD_OP_PROJ, inst, n);
    if (vs != DD_OK) return vs;
    if (!angles || !planp) return DD_ERR_INVALID_ARG;
    for (int i = 0; i < n; i++)
        if (!angles[i]) return DD_ERR_INVALID_ARG;
    BatchLayout L = batch_layout(scan, inst, n, kBI);
    if (plan_bytes < L.total) return DD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *pb = (char *)planp;
    // work items; longest first unless the tuning asks for instance order
    struct Item {
        int4 w;
        long long cost;
    };
    std::vector<Item> fw, aw;
    fw.reserve(L.nfwd);
    aw.reserve(L.nadj);
    for (int i = 0; i < n; i++) {
        const BatchInst &d = L.inst[i];
        const int W = d.g.width, H = d.g.height, D = d.g.num_det;
        for (int b0 = 0; b0 < d.batch; b0 += L.fi) {
            const int nb = std::min(L.fi, d.batch - b0);
            for (int v = 0; v < d.V; v++)
                fw.push_back({make_int4(i, v, b0, nb), (long long)std::max(W, H) * (D + 1) * nb});
        }
        for (int b0 = 0; b0 < d.batch; b0 += kBI) {
            const int nb = std::min(kBI, d.batch - b0);
            for (int ty = 0; ty < (H + kTile - 1) / kTile; ty++)
                for (int tx = 0; tx < (W + kTile - 1) / kTile; tx++)
                    aw.push_back({make_int4(i, tx | (ty << 16), b0, nb), (long long)d.V * nb});
        }
    }
    const bool lpt = !tune || tune->lpt_order != 0;
    if (lpt) {
        std::stable_sort(fw.begin(), fw.end(), [](const Item &a, const Item &b) { return a.cost > b.cost; });
        std::stable_sort(aw.begin(), aw.end(), [](const Item &a, const Item &b) { return a.cost > b.cost; });
    }
    std::vector<int4> fi(fw.size()), ai(aw.size());
    for (size_t k = 0; k < fw.size(); k++) fi[k] = fw[k].w;
    for (size_t k = 0; k < aw.size(); k++) ai[k] = aw[k].w;
    // descriptors and item lists (plan time only: synchronous copies)
    if (cudaMemcpyAsync(pb + L.desc, L.inst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(pb + L.fitems, fi.data(), sizeof(int4) * fi.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(pb + L.aitems, ai.data(), sizeof(int4) * ai.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return DD_ERR_LAUNCH;
    for (int i = 0; i < n; i++) {
        const BatchInst &d = L.inst[i];
        const int s2 = plan(scan, &d.g, angles[i], d.V, pb + L.plans + d.plan_off,
                            plan_layout(scan, &d.g, d.V).total, st);
        if (s2 != DD_OK) return s2;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return DD_ERR_LAUNCH;
    return DD_OK;
}

extern "C" int dd2d_batch_apply(int scan, int op, const dd_instance2d *inst, int n, const void *planp,
                                const float *in, float *out, void *ws, size_t wsb, const dd_tune2d *tune,
                                dd_stream_t stream) {
    ddtrace::Range tr("dd2d_batch_apply", scan, op, false);
    const int vs = validate_batch(scan, op, inst, n);
    if (vs != DD_OK) return vs;
    if (!planp || !in || !out) return DD_ERR_INVALID_ARG;
    const BatchLayout L = batch_layout(scan, inst, n, kBI);
    if (!ws || wsb < L.w_total) return DD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *wb = (char *)ws;
    if (cudaMemsetAsync(wb + L.w_status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    if (op_is_forward(op))
        return batch_forward(scan, op, L, (const char *)planp, in, out, nullptr, wb, tune, st);
    return batch_adjoint(scan, op, L, (const char *)planp, in, out, nullptr, 1.0f, wb, tune, st);
}

extern "C" int dd2d_batch_dc_step(int scan, const dd_instance2d *inst, int n, const void *planp, float *x,
                                  const float *y, float eta, void *ws, size_t wsb, const dd_tune2d *tune,
                                  dd_stream_t stream) {
    ddtrace::Range tr("dd2d_batch_dc_step", scan, -1, false);
    const int vs = validate_batch(scan, DD_OP_PROJ, inst, n);
    if (vs != DD_OK) return vs;
    if (!planp || !x || !y) return DD_ERR_INVALID_ARG;
    const BatchLayout L = batch_layout(scan, inst, n, kBI);
    if (!ws || wsb < L.w_total) return DD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *wb = (char *)ws;
    float *resid = (float *)(wb + L.w_resid);
    const char *pb = (const char *)planp;
    if (cudaMemsetAsync(wb + L.w_status, 0, sizeof(int), st) != cudaSuccess) return DD_ERR_LAUNCH;
    int s1 = batch_forward(scan, DD_OP_PROJ, L, pb, x, resid, y, wb, tune, st);
    if (s1 != DD_OK) return s1;
    return batch_adjoint(scan, DD_OP_PROJ_T, L, pb, resid, x, x, -eta, wb, tune, st);
}

int dd2b_set_sink(int *sink) { return dd_set_status_sink_tu(sink); }

extern "C" int dd2d_batch_status(int scan, const dd_instance2d *inst, int n, const void *ws, int *status) {
    if (validate_batch(scan, DD_OP_PROJ, inst, n) != DD_OK || !ws || !status) return DD_ERR_INVALID_ARG;
    const BatchLayout L = batch_layout(scan, inst, n, kBI);
    if (cudaMemcpy(status, (const char *)ws + L.w_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return DD_ERR_LAUNCH;
    return DD_OK;
}
