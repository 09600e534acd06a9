// Fan-flat forward projection for callers that cannot allocate device memory.
//
// Who needs this: code that runs where cudaMalloc is not an option -- a
// plugin whose host framework owns every byte of device memory and exposes
// no allocator to it, a real-time loop that must not touch the allocator
// once started, or a caller that has no place to keep a workspace between
// calls.  The regular entry points take their scratch from the caller
// (`workspace`); this one takes it from a buffer that is part of the
// library image itself.
//
// The buffer: `g_dd_noalloc_scratch`, a file-scope __device__ array of
// DD_NOALLOC_SCRATCH_BYTES (32 MiB).  Every GPU that loads the library keeps
// these 32 MiB until the process exits.  Problems whose plan and workspace
// need more than that are refused with DD_ERR_WORKSPACE before any work is
// enqueued (dd2d_workspace_bytes gives the need: roughly 592 bytes per
// (view, image line) plus the line tables, e.g. 256x256 images with 180
// views fit, 512x512 with 720 views do not).
//
// The first call on a device looks up the buffer's device address with
// cudaGetSymbolAddress, with that device current; make that first call
// before capturing a stream into a CUDA graph.  The address is kept for the
// life of the process: do not use this entry point on a device after
// cudaDeviceReset (or any other teardown of its primary context), which
// would leave the kept address pointing at freed memory.  A timeout of a
// bounded device-side wait is reported by dd_noalloc_status.  All calls share the one
// buffer: two calls whose work overlaps on the GPU (different streams, or
// different host threads, without ordering between them) race on it and
// produce garbage.  Each call rewrites everything it reads from the buffer
// (geometry plan, prefix tables, and a zeroed status word), so nothing left
// by the previous call leaks into the next.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pridediff_dd.h"

#define DD_NOALLOC_SCRATCH_BYTES (32u << 20)

static __device__ __align__(256) unsigned char g_dd_noalloc_scratch[DD_NOALLOC_SCRATCH_BYTES];

size_t dd2d_status_offset(int scan, int op, const dd_geom2d *g, int batch, int num_view);   // dd2d.cu

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_lock;
void *g_addr[kMaxDevices] = {};
size_t g_status_off[kMaxDevices] = {};   // status word of the last call on each device
bool g_called[kMaxDevices] = {};

// Device address of the scratch buffer on the current device (set-up on
// first use per device).  Returns nullptr if the lookup fails.
void *scratch_on_current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> hold(g_lock);
    if (!g_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_dd_noalloc_scratch) != cudaSuccess) return nullptr;
        g_addr[dev] = p;
    }
    return g_addr[dev];
}
}  // namespace

extern "C" int dd_ProjFanFlatDis2d_noalloc(const dd_geom2d *g, const float *in, float *out,
                                            const float *angles, int batch, int num_view,
                                            dd_stream_t stream) {
    const int st = dd2d_validate(DD_SCAN_FLAT, DD_OP_PROJ, g, batch, num_view);
    if (st != DD_OK) return st;
    if (!in || !out || !angles) return DD_ERR_INVALID_ARG;
    const size_t need = dd2d_workspace_bytes(DD_SCAN_FLAT, DD_OP_PROJ, g, batch, num_view);
    if (need == 0 || need > DD_NOALLOC_SCRATCH_BYTES) return DD_ERR_WORKSPACE;
    void *scratch = scratch_on_current_device();
    if (!scratch) return DD_ERR_LAUNCH;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DD_ERR_LAUNCH;
    {
        std::lock_guard<std::mutex> hold(g_lock);
        g_status_off[dev] = dd2d_status_offset(DD_SCAN_FLAT, DD_OP_PROJ, g, batch, num_view);
        g_called[dev] = true;
    }
    return dd2d_apply(DD_SCAN_FLAT, DD_OP_PROJ, g, in, out, angles, batch, num_view, scratch,
                      DD_NOALLOC_SCRATCH_BYTES, stream);
}

// Status word (DD_OK or DD_ERR_TIMEOUT) of the last call on the current
// device, copied from the library's buffer; synchronous.  DD_OK before any
// call.  A later call overwrites it.
extern "C" int dd_noalloc_status(int *status) {
    if (!status) return DD_ERR_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DD_ERR_LAUNCH;
    size_t off;
    {
        std::lock_guard<std::mutex> hold(g_lock);
        if (!g_called[dev]) {
            *status = DD_OK;
            return DD_OK;
        }
        off = g_status_off[dev];
    }
    if (cudaMemcpyFromSymbol(status, g_dd_noalloc_scratch, sizeof(int), off, cudaMemcpyDeviceToHost) != cudaSuccess)
        return DD_ERR_LAUNCH;
    return DD_OK;
}
