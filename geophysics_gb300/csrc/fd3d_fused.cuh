// Fused 3D VTI time step: shared declarations between the plan (fd3d.cu)
// and the y-marching TMA kernel (fd3d_fused.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace geo {

// Tensor maps of one step's reads.  Per time level: 0 P x-halo box, 1 P own
// box, 2 Q z-halo box, 3 u x-halo box, 4 w z-halo box, 5 v own box; then
// the level-independent own boxes 6-8 model, 9-14 split stresses.
constexpr int kNumMaps = 15;
struct StepMaps {
    CUtensorMap m[kNumMaps];
};

struct Fused3D {
    int nnx, nny, nnz, ldz;
    long sxy;
    int npd, nx, ny, nz;
    float dtx, dty, dtz;
    const float *cx1, *cx2, *ax1, *ax2, *cy1, *cy2, *ay1, *ay2, *cz1, *cz2, *az1, *az2;
    const float *m0, *m1, *m2;             // model: (vp, 1+2eps, sqrtf(1+2del)) exact,
                                           //        (A, B, C) fast
    const float *P0, *Q0;                  // current level (source cell)
    float *u1, *v1, *w1, *P1, *Q1;         // next level
    float *px, *py, *pz, *qx, *qy, *qz;    // split stresses (in place)
    int ntz, ntx, ntiles, chunk, nitems;   // work decomposition
    int *err;                              // device error word (wait timeouts)
};

// Tile and pipeline geometry.
constexpr int kTZ = 32;                 // z points per tile (one warp's lanes)
constexpr int kTXF = 16;                // x columns per tile (two per thread)
constexpr int kWarps = kTXF / 2;        // warps per block
constexpr int kStages = 3;              // TMA pipeline depth (planes)
constexpr int kPB = kTZ * (kTXF + 14);  // P x-halo box (z 32, x TX+14 from x0-7)
constexpr int kQB = 48 * kTXF;          // Q / w box (z 48 from z0-8, x TX)
constexpr int kUB = kTZ * (kTXF + 8);   // u box (z 32, x TX+8 from x0-4)
constexpr int kOB = kTZ * kTXF;         // own box (z 32, x TX)
// stage: P own (plane y+7), v (plane y+3), then the stress plane's P halo,
// Q, u, w, model (3) and split stresses (6)
constexpr int kStageFloats = kOB + kOB + kPB + kQB + kUB + kQB + 3 * kOB + 6 * kOB;
constexpr int kUTile = (kTXF + 7) * kTZ;
constexpr int kWTile = kTXF * 40;
constexpr size_t kFusedSmem = (size_t)(kStages * kStageFloats + kUTile + kWTile) * 4 + 256;

struct StepArgs3D;
int launch_fused3d(const StepMaps &maps, const Fused3D &g, int mode, const StepArgs3D &st, cudaStream_t s);
int encode_map(CUtensorMap *map, const float *base, int nnz, int ldz, int nnx, int nny, int boxz, int boxx);

}  // namespace geo
