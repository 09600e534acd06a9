// C-ABI shim over deeprecon's own CPU projectors (test infrastructure only).
//
// The Makefile in this directory compiles this file together with the
// reference sources deeprecon/cpu/dis2d/{Para,FanFlat,FanArc}DisCPU2d.cpp,
// unmodified and where they lie, into _ref/libddref.so.  The wrappers below
// only rename the entry points to extern "C" symbols so that ctypes can call
// them; every number they return is computed by the reference code.
//
// The signatures follow deeprecon/include/dis2d/*CPU2d.h (e.g.
// FanFlatDisCPU2d.h:3-22): (Image, Projection, ViewAngle, BatchSize, Width,
// Height, NumView, NumDet, ImageSizeX, ImageSizeY, DetSize, IsoSource,
// SourceDetector, PixXShift, PixYShift, BinShift).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ParaDisCPU2d.h"
#include "FanFlatDisCPU2d.h"
#include "FanArcDisCPU2d.h"

#define REF_ARGS                                                              \
    float *img, float *proj, float *ang, int batch, int w, int h, int nv,     \
        int nd, float sx, float sy, float ds, float r, float sdd, float px,   \
        float py, float bs
#define REF_PASS img, proj, ang, batch, w, h, nv, nd, sx, sy, ds, r, sdd, px, py, bs

#define WRAP(name) \
    extern "C" void ref_##name(REF_ARGS) { name(REF_PASS); }

WRAP(ProjParaDisCPU2d)
WRAP(ProjTransParaDisCPU2d)
WRAP(BackProjParaDisCPU2d)
WRAP(BackProjTransParaDisCPU2d)

WRAP(ProjFanFlatDisCPU2d)
WRAP(ProjTransFanFlatDisCPU2d)
WRAP(BackProjFanFlatDisCPU2d)
WRAP(BackProjTransFanFlatDisCPU2d)
WRAP(BackProjWeightedFanFlatDisCPU2d)
WRAP(BackProjTransWeightedFanFlatDisCPU2d)

WRAP(ProjFanArcDisCPU2d)
WRAP(ProjTransFanArcDisCPU2d)
WRAP(BackProjFanArcDisCPU2d)
WRAP(BackProjTransFanArcDisCPU2d)
WRAP(BackProjWeightedFanArcDisCPU2d)
WRAP(BackProjTransWeightedFanArcDisCPU2d)

// System-matrix builders (RadonTorch.cpp:1270-1372 call these).  The COO
// triplets are returned in malloc'd arrays that the caller releases with
// ref_free.  geom: 0 = parallel, 1 = fan-flat, 2 = fan-arc.
extern "C" int64_t ref_sysmatrix(int geom, const float *ang, int w, int h, int nv,
                                 int nd, float sx, float sy, float ds, float r,
                                 float sdd, float px, float py, float bs,
                                 int64_t **rows, int64_t **cols, float **vals) {
    std::vector<int64_t> i, j;
    std::vector<float> v;
    if (geom == 0)
        GetSysMatrixPara2dKernel(i, j, v, ang, w, h, nv, nd, sx, sy, ds, r, sdd, px, py, bs);
    else if (geom == 1)
        GetSysMatrixFanFlat2dKernel(i, j, v, ang, w, h, nv, nd, sx, sy, ds, r, sdd, px, py, bs);
    else
        GetSysMatrixFanArc2dKernel(i, j, v, ang, w, h, nv, nd, sx, sy, ds, r, sdd, px, py, bs);
    const int64_t n = (int64_t)v.size();
    *rows = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));
    *cols = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));
    *vals = (float *)malloc(sizeof(float) * (n ? n : 1));
    if (n) {
        memcpy(*rows, i.data(), sizeof(int64_t) * n);
        memcpy(*cols, j.data(), sizeof(int64_t) * n);
        memcpy(*vals, v.data(), sizeof(float) * n);
    }
    return n;
}

extern "C" void ref_free(void *p) { free(p); }
