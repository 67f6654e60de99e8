// Device-side views of a 3D grid, shared by the 3D kernels.
#pragma once
#include <cuda_runtime.h>

struct geo_fd3d_plan;

namespace geo {

struct Grid3D {
    int nnx, nny, nnz, ldz;     // padded extents; ldz = z stride (nnz rounded up to 4)
    long sxy;                   // y stride
    int npd, nx, ny, nz;        // sponge width and interior extents
    float dtx, dty, dtz;        // dt/dx etc. (float division, as the reference)
    const float *cx1, *cx2, *ax1, *ax2, *cy1, *cy2, *ay1, *ay2, *cz1, *cz2, *az1, *az2;
    const float *vp, *e2, *d2;  // vp, 1+2eps, sqrtf(1+2del)
    float *u, *v, *w, *P, *Q;
    float *px, *py, *pz, *qx, *qy, *qz;
};

struct StepArgs3D {
    int it;
    int src_on;
    float amp;
    int ixs, iys, izs;
    long src;                   // linear source index (or -1)
    float *rec;                 // time-major record (nt x nrx*nry) or null
    int rec_iz, rx0, drx, nrx, ry0, dry, nry;
    int rec_pq;                 // record P+Q instead of P (the 3D RTM program)
    float *ill;                 // interior illumination += P^2+Q^2 (or null)
    float *mig;                 // interior image += other_P * P (or null)
    const float *other_P;       // the source-side field's P (same layout)
};

// One 3D TTI step (tti3d.cu): g describes the grid, its profiles and the
// premultiplied model (vp, e2, d2 hold A, B, C); level c is read, level n
// written; ct..sp are cos/sin of tilt and azimuth; save keeps the source
// cell's P,Q of level c.
struct Tti3DStep {
    Grid3D g;
    const float *u0, *v0, *w0, *P0, *Q0;
    float *u1, *v1, *w1, *P1, *Q1;
    const float *ct, *st, *cp, *sp;
    float *save;
    int *err;                   // device error word (pipeline wait timeouts)
};
int launch_tti3d(const Tti3DStep &t, const StepArgs3D &st, cudaStream_t s);

Grid3D make_grid(const geo_fd3d_plan *p);
int run_shot_3d(geo_fd3d_plan *p, int is, cudaStream_t s, int (*on_step)(void *, int), void *ctx);
int fetch_shot_3d(geo_fd3d_plan *p, float *shot, int mem, cudaStream_t s);
int plan3d_dims(const geo_fd3d_plan *p, int *nnx, int *nny, int *nnz);

}  // namespace geo
