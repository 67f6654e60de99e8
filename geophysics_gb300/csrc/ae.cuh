// Learned snapshot codec: a 4-level convolutional autoencoder over 16^3
// blocks of a wavefield, kernel 2 = stride 2 at every level, so one block
// is coded independently of its neighbours and every level is a dense GEMM
// once the block's points are stored in Morton (bit-interleaved z,x,y)
// order: the 8 children of a level-l cell are then contiguous rows of the
// level-(l-1) output.
//
//   encoder                                     decoder
//   E1  8 pts     -> 16   leaky ReLU (CUDA)     D4  512  -> 8x256  leaky ReLU
//   E2  8x16      -> 64   leaky ReLU (tcgen05)  D3  256  -> 8x64   leaky ReLU
//   E3  8x64      -> 256  leaky ReLU (tcgen05)  D2  64   -> 8x16   leaky ReLU
//   E4  8x256     -> 512  linear     (tcgen05)  D1  16   -> 8 pts  linear (CUDA)
//
// A block is scaled by its max |value| before E1 and after D1; the code is
// 512 bf16 (1 KiB) plus one fp32 scale per 4096 fp32 points (16 KiB):
// 15.9x compression.  Weights and activations are bf16, accumulation fp32.
#pragma once
#include "geo_internal.h"
#include <cuda_bf16.h>

namespace geo {

constexpr int kAeBlock = 16;                 // block edge
constexpr int kAePts = 4096;                 // points per block
constexpr int kAeLat = 512;                  // latent width per block
constexpr int kAeLayers = 8;                 // E1 E2 E3 E4 D4 D3 D2 D1

// Layer l: out width N, in width K (per row), rows per block, activation.
struct AeLayer {
    int N, K, rows, act;
};
constexpr AeLayer kAeNet[kAeLayers] = {
    {16, 8, 512, 1},     // E1
    {64, 128, 64, 1},    // E2
    {256, 512, 8, 1},    // E3
    {512, 2048, 1, 0},   // E4
    {2048, 512, 1, 1},   // D4
    {512, 256, 8, 1},    // D3
    {128, 64, 64, 1},    // D2
    {8, 16, 512, 0},     // D1
};

// Interior box of a padded z-fastest field (the codec's view of a snapshot).
struct AeVolume {
    const float *src;          // padded field, or null
    long ldz, sxy;             // strides of the padded field
    int oz, ox, oy;            // interior origin
    int nz, nx, ny;            // interior extents
    int nbz, nbx, nby;         // blocks per axis (ragged edges read as zero)
};

AeVolume ae_volume(const float *src, long ldz, long sxy, int oz, int ox, int oy, int nz, int nx, int ny);
// Padded block count of a box (codes and scales are allocated per row).
int ae_code_rows(const AeVolume &v);
// Residual slots per snapshot for escaped blocks.
int ae_escape_cap(geo_ae *ae, const AeVolume &v);
// esc/res/count may be null (no escapes).
int ae_encode_volume(geo_ae *ae, const AeVolume &v, void *code, float *scale, int *esc, void *res, int *count,
                     cudaStream_t s);
// mode 0: write the decoded snapshot to dst (v's strides); mode 1: add
// w * snapshot * gP (v's strides) to the image mig (iz + nz*(ix + nx*iy)).
int ae_decode_volume(geo_ae *ae, const AeVolume &v, const void *code, const float *scale, const int *esc,
                     const void *res, int mode, float *dst, const float *gP, float *mig, float w, cudaStream_t s);
int ae_check_err(geo_ae *ae, cudaStream_t s);
// Record coded and escaped block counts of an RTM shot (geo_ae_stats).
void ae_note_run(geo_ae *ae, long long blocks, long long escaped);

}  // namespace geo
