/*
 * CPU oracle for the distance-driven projector -- TEST INFRASTRUCTURE.
 *
 * A restatement, in plain C, of deeprecon's DD projector algorithm
 * (deeprecon/cpu/dis2d/<geom>DisCPU2d.cpp for 2-D, deeprecon/cuda/dis3d/<geom>DisCUDA3d.cu for 3-D,
 * which has no CPU path in the reference).  It is compiled at FP32
 * ("ddo_f_*", reproducing the reference's FP32 rounding, the parity oracle
 * and the timed CPU "port") and at FP64 ("ddo_d_*", the FP64 oracle).
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark call
 * it.  The product library never links it.
 */
#ifndef DDORACLE_H
#define DDORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* geometries (deeprecon scan_type) */
enum { DDO_PARA = 0, DDO_FLAT = 1, DDO_ARC = 2 };
enum { DDO_CONE_FLAT = 0, DDO_CONE_ARC = 1, DDO_SPIRAL = 2 };

/* operators, named after the radontorch functions they restate
 * (RadonTorch.cpp:1375-1418) */
enum {
    DDO_PROJ = 0,     /* Proj*            : image -> sinogram, A         */
    DDO_PROJ_T = 1,   /* ProjTrans*       : sinogram -> image, A^T       */
    DDO_BPROJ = 2,    /* BackProj*        : sinogram -> image, DD-BP B   */
    DDO_BPROJ_T = 3,  /* BackProjTrans*   : image -> sinogram, B^T       */
    DDO_BPROJ_W = 4,  /* BackProjWeighted*: FBP-weighted DD-BP           */
    DDO_BPROJ_TW = 5  /* BackProjTransWeighted*                          */
};

/* 2-D geometry: the 11-entry options vector of projector2d
 * (deeprecon/deeprecon/torch/projector/projector.py:113). */
typedef struct {
    int width, height, nd, nv;
    double pix_x, pix_y, det_size, iso_source, source_detector;
    double pix_xshift, pix_yshift, bin_shift;
} ddo_geom2;

/* 3-D geometry: the 17-entry options vector of projector3d (projector.py:286)
 * and the 16-entry vector of projectorsp (projector.py:460, no z shift). */
typedef struct {
    int width, height, depth, ncol, nrow, nv;
    double pix_x, pix_y, pix_z, col_size, row_size, iso_source, source_detector;
    double pix_xshift, pix_yshift, pix_zshift, col_shift, row_shift;
} ddo_geom3;

int ddo_default_threads(int nv);

int ddo_f_ddo_run2d(const ddo_geom2 *g, int geom, int op, const float *angles,
                    const float *in, float *out, int batch, int nthreads);
int ddo_d_ddo_run2d(const ddo_geom2 *g, int geom, int op, const float *angles,
                    const double *in, double *out, int batch, int nthreads);

/* source_pos: (4, nv) rows [axial, d_radius, d_angle, d_axial] for the spiral
 * (RadonTorch.cpp:1040-1043); NULL otherwise. */
int ddo_f_ddo_run3d(const ddo_geom3 *g, int geom, int op, const float *angles,
                    const float *source_pos, const float *in, float *out, int batch,
                    int nthreads);
int ddo_d_ddo_run3d(const ddo_geom3 *g, int geom, int op, const float *angles,
                    const float *source_pos, const double *in, double *out, int batch,
                    int nthreads);

/* Start-index scan of deeprecon's CUDA kernels (see ddoracle_body.h): the
 * number of (view, 256-column block, line) walk starts whose detector or
 * pixel index lies within `margin` of rounding to -1.  0 means the case is
 * safe to run on the reference kernels. */
long long ddo_f_ddo_scan2d(const ddo_geom2 *g, int geom, const float *angles, double margin,
                           int *per_view);
long long ddo_f_ddo_scan3d(const ddo_geom3 *g, int geom, const float *angles,
                           const float *source_pos, double margin, int *per_view);

#ifdef __cplusplus
}
#endif
#endif
