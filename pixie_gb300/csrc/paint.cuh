// Shared between the paint kernels (paint.cu) and the host (abi.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pxg {

struct Mat9 {
  float m[9];  // vmath Mat3, column-major
};

// One gradient fill: kind 3 linear, 4 radial, 5 angular (PaintKind); the
// stops (r, g, b, a, position) are in device memory.
struct GradientArgs {
  int kind;
  int nstops;
  float opacity;
  float atx, aty, dx, dy, det;  // linear: handle 0, handle 1 - handle 0, |d|^2
  float m[9];                   // radial: the inverse gradient matrix (column-major)
  float cx, cy, gradientAngle;  // angular: centre and the edge's angle
};

void launch_gradient(uint32_t* img, long long W, long long H, const GradientArgs& g, const float* stops, int nsm,
                     cudaStream_t st);
void launch_apply_opacity(uint32_t* img, long long n, uint32_t o, int nsm, cudaStream_t st);
void launch_draw_correct(uint32_t* a, long long W, long long H, const uint32_t* b, long long bw, long long bh,
                         const Mat9& inv, int mode, bool tiled, const uint8_t* tbl, int nsm, cudaStream_t st);

}  // namespace pxg
