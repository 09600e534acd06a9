// Host launcher for deeprecon's own CUDA projector kernels -- TEST
// INFRASTRUCTURE (the checker and the "plain GPU" comparator; never the
// product).
//
// The device code is deeprecon's, unmodified: the Makefile in this directory
// compiles deeprecon/cuda/dis2d/*.cu and deeprecon/cuda/dis3d/*.cu, where they
// lie, into one fatbin per file under _ref/cuda/ (sm_103a device code only;
// a fatbin carries no host code, so the same file serves any host CPU).  This
// file is the host side that the reference's own launchers would be, written
// here because their host code cannot be built for every host that runs the
// GPU: it loads those fatbins with the driver API, finds each kernel by its
// name and launches it exactly as the reference's host functions do:
//
//  * kernels that read the image read it through a texture object over a
//    cudaArray of extent (W, H, B) in 2-D or (W, H, B*Depth) in 3-D, with
//    border addressing, point filtering and unnormalised coordinates,
//    created, filled by a device-to-device cudaMemcpy3D and destroyed on
//    every call (e.g. FanFlatDisCUDA2d.cu:777-815, ConeFlatDisCUDA3d.cu:1083-1122);
//  * the others read the sinogram through a plain pointer and accumulate
//    into a zeroed image with atomics (FanFlatDisCUDA2d.cu:820-845);
//  * 256 threads per block; grid (B, V, ceil(D/256)) in 2-D
//    (FanFlatDisCUDA2d.cu:807-808) and (B*V, Rows, ceil(Cols/256)) in 3-D
//    (ConeFlatDisCUDA3d.cu:1110-1111), on the legacy default stream.
//
// Operator -> kernel pairing, as radontorch's host functions make it:
//   Proj              Proj<G>Kernel                (texture of the image)
//   ProjTrans         ProjTrans<G>Kernel           (sinogram pointer)
//   BackProj          BackProj<G>Kernel<false>     (sinogram pointer)
//   BackProjTrans     BackProjTrans<G>Kernel<false>(texture)
//   BackProjWeighted  BackProj<G>Kernel<true>
//   BackProjTransWeighted BackProjTrans<G>Kernel<true>
// and for the parallel beam (ParaDisCUDA2d.cu:337, 368, 396, 452):
//   Proj -> ProjParaKernel<false>, ProjTrans -> BackProjParaKernel<true>,
//   BackProj -> BackProjParaKernel<false>, BackProjTrans -> ProjParaKernel<true>.
//
// Kernel arguments (e.g. ConeFlatDisCUDA3d.cu:27-49, SpiralDisCUDA3d.cu:34-58,
// FanFlatDisCUDA2d.cu:27-42): (output, input pointer or texture object,
// ViewAngle, [spiral: the four rows of SourcePos], then the integer sizes and
// the float geometry in the order of radontorch's options vector).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace {

enum Geom { PARA = 0, FLAT, ARC, CONE_FLAT, CONE_ARC, SPIRAL, NGEOM };
enum Op { PROJ = 0, PROJ_T, BPROJ, BPROJ_T, BPROJ_W, BPROJ_TW, NOP };

const char* kFile[NGEOM] = {"ParaDisCUDA2d", "FanFlatDisCUDA2d", "FanArcDisCUDA2d",
                            "ConeFlatDisCUDA3d", "ConeArcDisCUDA3d", "SpiralDisCUDA3d"};
const char* kTag[NGEOM] = {"Para", "FanFlat", "FanArc", "ConeFlat", "ConeArc", "Spiral"};

struct KernelSpec {
    std::string base;  // unmangled kernel name
    int tmpl;          // -1: not a template; 0/1: the bool template argument
    bool texture;      // reads the image through a texture object
};

bool spec_of(int g, int op, KernelSpec* s) {
    const bool d3 = g >= CONE_FLAT;
    const std::string suffix = std::string(kTag[g]) + (d3 ? "DisCUDA3dKernel" : "DisCUDA2dKernel");
    if (g == PARA) {
        switch (op) {
            case PROJ: *s = {"Proj" + suffix, 0, true}; return true;
            case PROJ_T: *s = {"BackProj" + suffix, 1, false}; return true;
            case BPROJ: *s = {"BackProj" + suffix, 0, false}; return true;
            case BPROJ_T: *s = {"Proj" + suffix, 1, true}; return true;
            default: return false;
        }
    }
    switch (op) {
        case PROJ: *s = {"Proj" + suffix, -1, true}; return true;
        case PROJ_T: *s = {"ProjTrans" + suffix, -1, false}; return true;
        case BPROJ: *s = {"BackProj" + suffix, 0, false}; return true;
        case BPROJ_T: *s = {"BackProjTrans" + suffix, 0, true}; return true;
        case BPROJ_W: *s = {"BackProj" + suffix, 1, false}; return true;
        case BPROJ_TW: *s = {"BackProjTrans" + suffix, 1, true}; return true;
        default: return false;
    }
}

std::mutex g_mu;
std::string g_err;
CUmodule g_mod[NGEOM] = {};
CUcontext g_ctx = nullptr;
CUfunction g_fn[NGEOM][NOP] = {};

int fail(const std::string& msg) {
    g_err = msg;
    return 1;
}

int fail_cu(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    return fail(std::string(what) + ": " + (s ? s : "unknown driver error"));
}

int fail_rt(const char* what, cudaError_t e) {
    return fail(std::string(what) + ": " + cudaGetErrorString(e));
}

// The Itanium-mangled name of `base` starts with "_Z<len><base>"; a template
// instance continues with "ILb0E" / "ILb1E".  Matching that prefix picks one
// kernel among a file's kernels without spelling out parameter mangling.
bool name_matches(const char* mangled, const KernelSpec& s) {
    std::string pre = "_Z" + std::to_string(s.base.size()) + s.base;
    if (std::strncmp(mangled, pre.c_str(), pre.size()) != 0) return false;
    const char* rest = mangled + pre.size();
    if (s.tmpl < 0) return rest[0] != 'I';
    return std::strncmp(rest, s.tmpl ? "ILb1E" : "ILb0E", 5) == 0;
}

int resolve(int g, int op, CUfunction* out) {
    if (g_fn[g][op]) {
        *out = g_fn[g][op];
        return 0;
    }
    KernelSpec s;
    if (!spec_of(g, op, &s)) return fail("operator not provided by the reference for this geometry");
    unsigned int n = 0;
    CUresult r = cuModuleGetFunctionCount(&n, g_mod[g]);
    if (r != CUDA_SUCCESS) return fail_cu("cuModuleGetFunctionCount", r);
    std::vector<CUfunction> fns(n);
    r = cuModuleEnumerateFunctions(fns.data(), n, g_mod[g]);
    if (r != CUDA_SUCCESS) return fail_cu("cuModuleEnumerateFunctions", r);
    CUfunction hit = nullptr;
    int hits = 0;
    for (CUfunction f : fns) {
        const char* nm = nullptr;
        if (cuFuncGetName(&nm, f) != CUDA_SUCCESS || !nm) continue;
        if (name_matches(nm, s)) {
            hit = f;
            ++hits;
        }
    }
    if (hits != 1)
        return fail("kernel " + s.base + (s.tmpl < 0 ? "" : (s.tmpl ? "<true>" : "<false>")) +
                    " found " + std::to_string(hits) + " times in " + kFile[g]);
    g_fn[g][op] = hit;
    *out = hit;
    return 0;
}

}  // namespace

extern "C" {

const char* refcuda_last_error() { return g_err.c_str(); }

// Loads <dir>/<file>.fatbin for every geometry into the current device's
// primary context.  Returns 0 on success.
int refcuda_load(const char* dir) {
    std::lock_guard<std::mutex> lk(g_mu);
    cudaError_t e = cudaFree(nullptr);  // make the runtime's primary context current
    if (e != cudaSuccess) return fail_rt("cudaFree(0)", e);
    CUcontext ctx = nullptr;
    CUresult r = cuCtxGetCurrent(&ctx);
    if (r != CUDA_SUCCESS || !ctx) return fail_cu("cuCtxGetCurrent", r);
    if (g_ctx == ctx && g_mod[0]) return 0;
    for (int g = 0; g < NGEOM; ++g) {
        std::string path = std::string(dir) + "/" + kFile[g] + ".fatbin";
        CUmodule m = nullptr;
        r = cuModuleLoad(&m, path.c_str());
        if (r != CUDA_SUCCESS) return fail_cu(("cuModuleLoad " + path).c_str(), r);
        g_mod[g] = m;
        for (int op = 0; op < NOP; ++op) g_fn[g][op] = nullptr;
    }
    g_ctx = ctx;
    return 0;
}

// One reference operator call.  `out` must be zeroed by the caller for the
// accumulating operators (ProjTrans, BackProj, BackProjWeighted), as
// radontorch allocates them with torch::zeros.  ints: W, H, NumView, NumDet
// (2-D) or W, H, Depth, NumView, NumDetCol, NumDetRow (3-D); floats: the
// geometry floats in the order of the reference kernel's parameters (8 in
// 2-D, 12 for cone, 11 for spiral).  `source_pos` is the (4, V) spiral table.
int refcuda_run(int geom, int op, float* out, const float* in, const float* angles,
                const float* source_pos, int batch, const int* ints, const float* floats) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (geom < 0 || geom >= NGEOM || op < 0 || op >= NOP) return fail("bad geometry or operator");
    if (!g_mod[geom]) return fail("refcuda_load has not been called");
    KernelSpec s;
    if (!spec_of(geom, op, &s)) return fail("operator not provided by the reference for this geometry");
    CUfunction fn;
    if (resolve(geom, op, &fn)) return 1;
    const bool d3 = geom >= CONE_FLAT;
    const int W = ints[0], H = ints[1];
    const int depth = d3 ? ints[2] : 1;
    const int nview = d3 ? ints[3] : ints[2];
    const int ncol = d3 ? ints[4] : ints[3];
    const int nrow = d3 ? ints[5] : 1;

    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    if (s.texture) {
        cudaChannelFormatDesc cd = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
        cudaExtent ext = make_cudaExtent((size_t)W, (size_t)H, (size_t)batch * depth);
        cudaError_t e = cudaMalloc3DArray(&arr, &cd, ext);
        if (e != cudaSuccess) return fail_rt("cudaMalloc3DArray", e);
        cudaMemcpy3DParms cp;
        std::memset(&cp, 0, sizeof(cp));
        cp.extent = ext;
        cp.kind = cudaMemcpyDeviceToDevice;
        cp.srcPtr = make_cudaPitchedPtr((void*)in, ext.width * sizeof(float), ext.width, ext.height);
        cp.dstArray = arr;
        e = cudaMemcpy3D(&cp);
        if (e != cudaSuccess) {
            cudaFreeArray(arr);
            return fail_rt("cudaMemcpy3D", e);
        }
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
        if (e != cudaSuccess) {
            cudaFreeArray(arr);
            return fail_rt("cudaCreateTextureObject", e);
        }
    }

    // argument block: pointers to each kernel argument, in parameter order
    float* a_out = out;
    const float* a_in = in;
    const float* a_ang = angles;
    const float* a_sp[4] = {nullptr, nullptr, nullptr, nullptr};
    int a_int[6];
    float a_flt[12];
    std::vector<void*> args;
    args.push_back(&a_out);
    if (s.texture) args.push_back(&tex);
    else args.push_back(&a_in);
    args.push_back(&a_ang);
    if (geom == SPIRAL) {
        for (int r = 0; r < 4; ++r) {
            a_sp[r] = source_pos + (size_t)r * nview;
            args.push_back(&a_sp[r]);
        }
    }
    const int nint = d3 ? 6 : 4;
    const int nflt = geom == SPIRAL ? 11 : (d3 ? 12 : 8);
    for (int i = 0; i < nint; ++i) {
        a_int[i] = ints[i];
        args.push_back(&a_int[i]);
    }
    for (int i = 0; i < nflt; ++i) {
        a_flt[i] = floats[i];
        args.push_back(&a_flt[i]);
    }

    const unsigned nblk = (unsigned)((ncol - 1) / 256 + 1);
    unsigned gx, gy;
    if (d3) {
        gx = (unsigned)batch * (unsigned)nview;
        gy = (unsigned)nrow;
    } else {
        gx = (unsigned)batch;
        gy = (unsigned)nview;
    }
    CUresult r = cuLaunchKernel(fn, gx, gy, nblk, 256, 1, 1, 0, nullptr, args.data(), nullptr);
    int rc = 0;
    if (r != CUDA_SUCCESS) rc = fail_cu("cuLaunchKernel", r);
    if (s.texture) {
        cudaDestroyTextureObject(tex);
        cudaFreeArray(arr);
    }
    return rc;
}

}  // extern "C"
