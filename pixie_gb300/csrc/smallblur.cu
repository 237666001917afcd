// Gaussian blur passes for radii 1..8 on the CUDA cores.
//
// One pass of pixie's blur (images.nim:304-365) is, per channel,
//   out[x] = (sum_t w[t] * p[x - r + t]) div 256 div 255,   t = 0 .. 2r,
// with taps outside the image reading the outOfBounds colour.  For small
// radii the pass is memory-bound once each input pixel is touched once per
// thread: a thread computes 8 consecutive outputs along the pass axis from
// its 8 + 2r inputs, converting every input to float once (the byte under the
// exponent of 2^23, minus 2^23: exact) and accumulating channel pairs with
// packed f32x2 fused multiply-adds.  Every product (<= 255 * 65535) and every
// partial sum (< 2^24) is an integer that float32 holds exactly, so the sums
// are the reference's uint32 sums.  The quotient floor(S / 65280) is one
// packed FMA rounding toward minus infinity, S * C + 1.5 * 2^23 with
// C = 1/65280 rounded up to float32 (exact for every S < 2^24, checked
// exhaustively on the host), which leaves it in the low byte.
//
// X pass: threads take 8-pixel groups of a row (consecutive threads,
// consecutive groups; 16-byte loads and stores when rows are 16-byte
// aligned).  Y pass: threads take 8-row strips of one column (consecutive
// threads, consecutive columns: every load and store of a warp is 128
// contiguous bytes).  Rows or strips come from blockIdx.y, so a thread's
// coordinates cost no division; interior strips walk a pointer without
// bounds tests.  The radius is a template parameter, so the taps unroll
// and the X pass's aligned-load offset is a constant.
#include <algorithm>
#include <cstdint>

#include "pxg_device.cuh"

namespace pxg {

void note_launch();

namespace {

constexpr int kOut = 8;                            // outputs per thread along the pass
constexpr float kQuotC = 0x1.010102p-16f;          // RU(1/65280)
constexpr float kMagic = 12582912.0f;              // 1.5 * 2^23
constexpr float kBias = 8388608.0f;                // 2^23

__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  return ((uint64_t)__float_as_uint(hi) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// floor(S / 65280) of both lanes, in the low byte of each 32-bit half
__device__ __forceinline__ uint64_t f2_quot(uint64_t s, uint64_t kq, uint64_t km) {
  uint64_t d;
  asm("fma.rm.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(s), "l"(kq), "l"(km));
  return d;
}
// channels (r, g) and (b, a) of a pixel as exact float pairs
__device__ __forceinline__ void px_f2(uint32_t p, uint64_t nb, uint64_t& rg, uint64_t& ba) {
  const uint32_t r = __byte_perm(p, 0x4B000000u, 0x7650u), g = __byte_perm(p, 0x4B000000u, 0x7651u);
  const uint32_t b = __byte_perm(p, 0x4B000000u, 0x7652u), a = __byte_perm(p, 0x4B000000u, 0x7653u);
  rg = f2_add(((uint64_t)g << 32) | r, nb);
  ba = f2_add(((uint64_t)a << 32) | b, nb);
}
__device__ __forceinline__ uint32_t quot_px(uint64_t rg, uint64_t ba, uint64_t kq, uint64_t km) {
  const uint64_t q0 = f2_quot(rg, kq, km), q1 = f2_quot(ba, kq, km);
  const uint32_t lo = __byte_perm((uint32_t)q0, (uint32_t)(q0 >> 32), 0x0040u);  // [r, g, ., .]
  const uint32_t hi = __byte_perm((uint32_t)q1, (uint32_t)(q1 >> 32), 0x0040u);  // [b, a, ., .]
  return __byte_perm(lo, hi, 0x5410u);
}

template <int R>
__global__ void __launch_bounds__(256) k_blur_sx(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                 int W, int H, const uint16_t* __restrict__ kern, uint32_t oob,
                                                 int vec) {
  constexpr int NI = kOut + 2 * R;      // inputs per thread
  constexpr int D = (4 - (R & 3)) & 3;  // (x0 - R) mod 4, x0 a multiple of 8
  constexpr int NC = (D + NI + 3) / 4;  // 16-byte chunks covering them
  pdl_trigger();
  pdl_wait();
  uint64_t w2[2 * R + 1];
#pragma unroll
  for (int t = 0; t <= 2 * R; t++) {
    const float w = (float)kern[t];
    w2[t] = f2_pack(w, w);
  }
  const uint64_t nb = f2_pack(-kBias, -kBias), kq = f2_pack(kQuotC, kQuotC), km = f2_pack(kMagic, kMagic);
  const int gpr = (W + kOut - 1) / kOut;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  for (int y = blockIdx.y; y < H && g < gpr; y += gridDim.y) {  // one 8-pixel group of a row per thread
    const int x0 = g * kOut;
    const int xa = x0 - R - D;  // 16-byte aligned when rows are
    const uint32_t* row = in + (long long)y * W;
    uint32_t px[4 * NC];
    if (vec && xa >= 0 && xa + 4 * NC <= W) {
#pragma unroll
      for (int c = 0; c < NC; c++) {
        const uint4 v = __ldcs(reinterpret_cast<const uint4*>(row + xa) + c);
        px[4 * c] = v.x;
        px[4 * c + 1] = v.y;
        px[4 * c + 2] = v.z;
        px[4 * c + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4 * NC; i++) {
        const int x = xa + i;
        px[i] = (x >= 0 && x < W) ? __ldcs(row + x) : oob;
      }
    }
    uint64_t arg[kOut], aba[kOut];
#pragma unroll
    for (int o = 0; o < kOut; o++) arg[o] = aba[o] = 0;
#pragma unroll
    for (int t = 0; t < NI; t++) {
      uint64_t rg, ba;
      px_f2(px[D + t], nb, rg, ba);
#pragma unroll
      for (int o = 0; o < kOut; o++) {
        if (t - o >= 0 && t - o <= 2 * R) {
          arg[o] = f2_fma(rg, w2[t - o], arg[o]);
          aba[o] = f2_fma(ba, w2[t - o], aba[o]);
        }
      }
    }
    uint32_t res[kOut];
#pragma unroll
    for (int o = 0; o < kOut; o++) res[o] = quot_px(arg[o], aba[o], kq, km);
    uint32_t* orow = out + (long long)y * W;
    if (vec && x0 + kOut <= W) {
      reinterpret_cast<uint4*>(orow + x0)[0] = make_uint4(res[0], res[1], res[2], res[3]);
      reinterpret_cast<uint4*>(orow + x0)[1] = make_uint4(res[4], res[5], res[6], res[7]);
    } else {
#pragma unroll
      for (int o = 0; o < kOut; o++)
        if (x0 + o < W) orow[x0 + o] = res[o];
    }
  }
}

template <int R>
__global__ void __launch_bounds__(256) k_blur_sy(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                 int W, int H, const uint16_t* __restrict__ kern, uint32_t oob) {
  constexpr int NI = kOut + 2 * R;
  pdl_trigger();
  pdl_wait();
  uint64_t w2[2 * R + 1];
#pragma unroll
  for (int t = 0; t <= 2 * R; t++) {
    const float w = (float)kern[t];
    w2[t] = f2_pack(w, w);
  }
  const uint64_t nb = f2_pack(-kBias, -kBias), kq = f2_pack(kQuotC, kQuotC), km = f2_pack(kMagic, kMagic);
  const int strips = (H + kOut - 1) / kOut;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  for (int s = blockIdx.y; s < strips && x < W; s += gridDim.y) {  // one 8-row strip of a column per thread
    const int y0 = s * kOut;
    uint32_t px[NI];
    if (y0 - R >= 0 && y0 + kOut + R <= H) {
      const uint32_t* p = in + (long long)(y0 - R) * W + x;
#pragma unroll
      for (int t = 0; t < NI; t++, p += W) px[t] = __ldcs(p);
    } else {
#pragma unroll
      for (int t = 0; t < NI; t++) {
        const int y = y0 - R + t;
        px[t] = (y >= 0 && y < H) ? __ldcs(in + (long long)y * W + x) : oob;
      }
    }
    uint64_t arg[kOut], aba[kOut];
#pragma unroll
    for (int o = 0; o < kOut; o++) arg[o] = aba[o] = 0;
#pragma unroll
    for (int t = 0; t < NI; t++) {
      uint64_t rg, ba;
      px_f2(px[t], nb, rg, ba);
#pragma unroll
      for (int o = 0; o < kOut; o++) {
        if (t - o >= 0 && t - o <= 2 * R) {
          arg[o] = f2_fma(rg, w2[t - o], arg[o]);
          aba[o] = f2_fma(ba, w2[t - o], aba[o]);
        }
      }
    }
    uint32_t* q = out + (long long)y0 * W + x;
#pragma unroll
    for (int o = 0; o < kOut; o++, q += W)
      if (y0 + o < H) __stcs(q, quot_px(arg[o], aba[o], kq, km));
  }
}

// Both passes in one launch, out of place (in -> out), for images the caller
// can swap: a CTA owns a TW x TH output tile; it runs the X pass over the
// tile's TH + 2R rows (rows outside the image hold the outOfBounds colour, as
// the Y pass's taps read it there), keeps the quantised bytes in shared
// memory, then runs the Y pass from shared memory and writes the tile once.
// DRAM traffic is one read and one write of the image (the halo rows shared
// by vertical neighbours come from L2).  The arithmetic per output is the
// two-pass kernels': the same sums, the same floor(S / 65280) between passes.
constexpr int kFTW = 128, kFTH = 64;  // tile: 128 columns x 64 rows
template <int R>
__global__ void __launch_bounds__(256) k_blur_fused(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                    int W, int H, const uint16_t* __restrict__ kern, uint32_t oob,
                                                    int vec, int late) {
  constexpr int NI = kOut + 2 * R;
  constexpr int D = (4 - (R & 3)) & 3;
  constexpr int NC = (D + NI + 3) / 4;
  constexpr int ROWS = kFTH + 2 * R;  // X-pass rows staged
  __shared__ __align__(16) uint32_t xs[ROWS][kFTW];
  if (late) pdl_trigger();  // else after the start-wait (pdl_late_entry)
  uint64_t w2[2 * R + 1];
#pragma unroll
  for (int t = 0; t <= 2 * R; t++) {
    const float w = (float)kern[t];
    w2[t] = f2_pack(w, w);
  }
  const uint64_t nb = f2_pack(-kBias, -kBias), kq = f2_pack(kQuotC, kQuotC), km = f2_pack(kMagic, kMagic);
  const int tx0 = blockIdx.x * kFTW, ty0 = blockIdx.y * kFTH;
  if (!late) pdl_late_entry(0);
  // X pass: (row, 8-pixel group) tasks over the staged rows
  constexpr int GPR = kFTW / kOut;  // groups per staged row
  for (int task = threadIdx.x; task < ROWS * GPR; task += blockDim.x) {
    const int lr = task / GPR, g = task - lr * GPR;
    const int y = ty0 - R + lr;
    const int x0 = tx0 + g * kOut;
    uint32_t res[kOut];
    if (y < 0 || y >= H) {
#pragma unroll
      for (int o = 0; o < kOut; o++) res[o] = oob;
    } else {
      const int xa = x0 - R - D;
      const uint32_t* row = in + (long long)y * W;
      uint32_t px[4 * NC];
      if (vec && xa >= 0 && xa + 4 * NC <= W) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
          const uint4 v = __ldg(reinterpret_cast<const uint4*>(row + xa) + c);
          px[4 * c] = v.x;
          px[4 * c + 1] = v.y;
          px[4 * c + 2] = v.z;
          px[4 * c + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 4 * NC; i++) {
          const int x = xa + i;
          px[i] = (x >= 0 && x < W) ? __ldg(row + x) : oob;
        }
      }
      uint64_t arg[kOut], aba[kOut];
#pragma unroll
      for (int o = 0; o < kOut; o++) arg[o] = aba[o] = 0;
#pragma unroll
      for (int t = 0; t < NI; t++) {
        uint64_t rg, ba;
        px_f2(px[D + t], nb, rg, ba);
#pragma unroll
        for (int o = 0; o < kOut; o++) {
          if (t - o >= 0 && t - o <= 2 * R) {
            arg[o] = f2_fma(rg, w2[t - o], arg[o]);
            aba[o] = f2_fma(ba, w2[t - o], aba[o]);
          }
        }
      }
#pragma unroll
      for (int o = 0; o < kOut; o++) res[o] = quot_px(arg[o], aba[o], kq, km);
    }
    uint4* dst = reinterpret_cast<uint4*>(&xs[lr][g * kOut]);
    dst[0] = make_uint4(res[0], res[1], res[2], res[3]);
    dst[1] = make_uint4(res[4], res[5], res[6], res[7]);
  }
  __syncthreads();
  // Y pass: (column, 8-row strip) tasks, consecutive threads on consecutive columns
  constexpr int STRIPS = kFTH / kOut;
  for (int task = threadIdx.x; task < STRIPS * kFTW; task += blockDim.x) {
    const int sidx = task / kFTW, c = task - sidx * kFTW;
    const int x = tx0 + c, y0 = ty0 + sidx * kOut;
    if (x >= W || y0 >= H) continue;
    uint64_t arg[kOut], aba[kOut];
#pragma unroll
    for (int o = 0; o < kOut; o++) arg[o] = aba[o] = 0;
#pragma unroll
    for (int t = 0; t < NI; t++) {
      uint64_t rg, ba;
      px_f2(xs[sidx * kOut + t][c], nb, rg, ba);
#pragma unroll
      for (int o = 0; o < kOut; o++) {
        if (t - o >= 0 && t - o <= 2 * R) {
          arg[o] = f2_fma(rg, w2[t - o], arg[o]);
          aba[o] = f2_fma(ba, w2[t - o], aba[o]);
        }
      }
    }
    uint32_t* q = out + (long long)y0 * W + x;
#pragma unroll
    for (int o = 0; o < kOut; o++, q += W)
      if (y0 + o < H) __stcs(q, quot_px(arg[o], aba[o], kq, km));
  }
  pdl_late_exit(late);
}

template <int R>
void launch_fused(const uint32_t* in, uint32_t* out, int W, int H, const uint16_t* kern, uint32_t oob,
                  cudaStream_t st) {
  const int vec = (W % 4 == 0) && ((reinterpret_cast<uintptr_t>(in) & 15) == 0);
  const dim3 grid((unsigned)((W + kFTW - 1) / kFTW), (unsigned)((H + kFTH - 1) / kFTH));
  const size_t bytes = (size_t)W * (size_t)H * 4;
  const int late = dep_late(st, {Span{out, bytes}}, {Span{in, bytes}});
  launch_pdl(k_blur_fused<R>, grid, dim3(256), 0, st, in, out, W, H, kern, oob, vec, late);
  note_launch();
}

template <int R>
void launch_small(uint32_t* img, uint32_t* tmp, int W, int H, const uint16_t* kern, uint32_t oob, int nsm,
                  cudaStream_t st) {
  const int vec = (W % 4 == 0) && ((reinterpret_cast<uintptr_t>(img) | reinterpret_cast<uintptr_t>(tmp)) & 15) == 0;
  // grids: x (blocks of 256 groups or columns) by rows or strips (capped; the
  // kernels loop over the rest)
  const unsigned gxx = (unsigned)(((W + kOut - 1) / kOut + 255) / 256), gxy = (unsigned)std::min(H, 65535);
  const unsigned gyx = (unsigned)((W + 255) / 256), gyy = (unsigned)std::min((H + kOut - 1) / kOut, 65535);
  launch_pdl(k_blur_sx<R>, dim3(gxx, gxy), dim3(256), 0, st, img, tmp, W, H, kern, oob, vec);
  note_launch();
  launch_pdl(k_blur_sy<R>, dim3(gyx, gyy), dim3(256), 0, st, tmp, img, W, H, kern, oob);
  note_launch();
}

}  // namespace

// Both passes in one launch, in -> out (out must not overlap in), for radii
// 1..8; false if r is not for this kernel.
bool launch_blur_small_fused(const uint32_t* in, uint32_t* out, long long W, long long H, int r,
                             const uint16_t* kern, uint32_t oob, cudaStream_t st) {
  if (r < 1 || r > 8 || W < 1 || H < 1 || W > (1 << 26) || H > (1 << 26)) return false;
  if ((H + kFTH - 1) / kFTH > 65535) return false;
  switch (r) {
    case 1: launch_fused<1>(in, out, (int)W, (int)H, kern, oob, st); break;
    case 2: launch_fused<2>(in, out, (int)W, (int)H, kern, oob, st); break;
    case 3: launch_fused<3>(in, out, (int)W, (int)H, kern, oob, st); break;
    case 4: launch_fused<4>(in, out, (int)W, (int)H, kern, oob, st); break;
    case 5: launch_fused<5>(in, out, (int)W, (int)H, kern, oob, st); break;
    case 6: launch_fused<6>(in, out, (int)W, (int)H, kern, oob, st); break;
    case 7: launch_fused<7>(in, out, (int)W, (int)H, kern, oob, st); break;
    default: launch_fused<8>(in, out, (int)W, (int)H, kern, oob, st); break;
  }
  return true;
}

// Both passes (img -> tmp -> img) for radii 1..kSmallBlurMax; false if r is
// not for these kernels.
constexpr int kSmallBlurMax = 8;
bool launch_blur_small(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                       uint32_t oob, int nsm, cudaStream_t st) {
  if (r < 1 || r > kSmallBlurMax || W < 1 || H < 1 || W > (1 << 26) || H > (1 << 26)) return false;
  switch (r) {
    case 1: launch_small<1>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    case 2: launch_small<2>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    case 3: launch_small<3>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    case 4: launch_small<4>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    case 5: launch_small<5>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    case 6: launch_small<6>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    case 7: launch_small<7>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
    default: launch_small<8>(img, tmp, (int)W, (int)H, kern, oob, nsm, st); break;
  }
  return true;
}

}  // namespace pxg
