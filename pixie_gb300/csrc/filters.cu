// Separable filters: gaussian blur (src/pixie/images.nim:304-365), spread
// (images.nim:700-758) and shadow (images.nim:760-776).
//
// blur: the X pass quantises each channel to uint8 (v div 256 div 255) before
// the Y pass, exactly as the reference's transposed intermediate does; taps
// outside the image take the outOfBounds colour.  Sums are exact uint32
// (255 * sum(weights) < 2^24).  Both passes stage a tile plus its halo in
// shared memory and run one output pixel per thread.
// shadow: MaskBlend reads only the mask's alpha and spread writes
// rgbx(0,0,0,v), so the whole shadow runs on one uint8 alpha plane.
#include "pxg_device.cuh"

namespace pxg {

void note_launch();

constexpr int kBX = 256;       // X pass: outputs per CTA
constexpr int kTX = 32;        // Y pass: tile width
constexpr int kTY = 64;        // Y pass: tile height
constexpr int kYThreadsY = 8;  // Y pass: block is 32 x 8

__device__ __forceinline__ void mac4(uint32_t s[4], uint32_t p, uint32_t w) {
  s[0] += (p & 255u) * w;
  s[1] += ((p >> 8) & 255u) * w;
  s[2] += ((p >> 16) & 255u) * w;
  s[3] += (p >> 24) * w;
}
__device__ __forceinline__ uint32_t quant4(const uint32_t s[4]) {
  return pack(s[0] / 256 / 255, s[1] / 256 / 255, s[2] / 256 / 255, s[3] / 256 / 255);
}

// ---- RGBX blur --------------------------------------------------------------
__global__ void __launch_bounds__(kBX) k_blur_x(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                long long W, long long H, int r,
                                                const uint16_t* __restrict__ kern, uint32_t oob) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* px = reinterpret_cast<uint32_t*>(sm);
  uint16_t* kw = reinterpret_cast<uint16_t*>(px + kBX + 2 * r);
  const long long y = blockIdx.y, x0 = (long long)blockIdx.x * kBX;
  const uint32_t* row = in + y * W;
  for (int i = threadIdx.x; i < kBX + 2 * r; i += kBX) {
    long long gx = x0 - r + i;
    px[i] = (gx >= 0 && gx < W) ? row[gx] : oob;
  }
  for (int i = threadIdx.x; i < 2 * r + 1; i += kBX) kw[i] = kern[i];
  __syncthreads();
  const long long x = x0 + threadIdx.x;
  if (x >= W) return;
  uint32_t s[4] = {0, 0, 0, 0};
  for (int k = 0; k <= 2 * r; k++) mac4(s, px[threadIdx.x + k], kw[k]);
  out[y * W + x] = quant4(s);
}

__global__ void __launch_bounds__(kTX * kYThreadsY) k_blur_y(const uint32_t* __restrict__ in,
                                                             uint32_t* __restrict__ out, long long W,
                                                             long long H, int r,
                                                             const uint16_t* __restrict__ kern,
                                                             uint32_t oob) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* px = reinterpret_cast<uint32_t*>(sm);  // (kTY + 2r) x kTX
  uint16_t* kw = reinterpret_cast<uint16_t*>(px + (kTY + 2 * r) * kTX);
  const long long x0 = (long long)blockIdx.x * kTX, y0 = (long long)blockIdx.y * kTY;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
  const long long x = x0 + tx;
  for (int i = ty; i < kTY + 2 * r; i += kYThreadsY) {
    long long gy = y0 - r + i;
    uint32_t v = oob;
    if (gy >= 0 && gy < H) v = x < W ? in[gy * W + x] : 0u;
    px[i * kTX + tx] = v;
  }
  for (int i = tid; i < 2 * r + 1; i += kTX * kYThreadsY) kw[i] = kern[i];
  __syncthreads();
  if (x >= W) return;
  for (int oy = ty; oy < kTY; oy += kYThreadsY) {
    long long y = y0 + oy;
    if (y >= H) break;
    uint32_t s[4] = {0, 0, 0, 0};
    for (int k = 0; k <= 2 * r; k++) mac4(s, px[(oy + k) * kTX + tx], kw[k]);
    out[y * W + x] = quant4(s);
  }
}


// ---- RGBX blur, float32 path ------------------------------------------------
// Every tap product and every partial sum is an integer below 2^24
// (255 * sum(weights) <= 255 * 65345), so float32 multiply-adds give the
// exact uint32 sums of the reference.  Pixels are staged in shared memory as
// float4 (converted once per load) and each thread accumulates one output
// with one 128-bit shared load and four FFMAs per tap.
constexpr int kFX = 256;             // X pass: outputs per row per CTA
constexpr int kFXRows = 2;           // X pass: rows per CTA
constexpr int kFYT = 64;             // Y pass: output rows per CTA
constexpr int kFYThreads = 8;        // Y pass: block is 32 x 8

__device__ __forceinline__ float4 px4(uint32_t p) {
  return make_float4((float)(p & 255u), (float)((p >> 8) & 255u), (float)((p >> 16) & 255u),
                     (float)(p >> 24));
}
__device__ __forceinline__ uint32_t quantf(float4 s) {  // v div 256 div 255 of the exact sums
  return pack((uint32_t)s.x / 65280u, (uint32_t)s.y / 65280u, (uint32_t)s.z / 65280u,
              (uint32_t)s.w / 65280u);
}

__global__ void __launch_bounds__(kFX) k_blurf_x(const uint32_t* __restrict__ in,
                                                 uint32_t* __restrict__ out, long long W,
                                                 long long H, int r,
                                                 const uint16_t* __restrict__ kern, uint32_t oob) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int span = kFX + 2 * r;
  float4* px = reinterpret_cast<float4*>(sm);                 // kFXRows x span
  float* kw = reinterpret_cast<float*>(px + kFXRows * span);  // 2r + 1
  const long long x0 = (long long)blockIdx.x * kFX, y0 = (long long)blockIdx.y * kFXRows;
  const float4 o = px4(oob);
  for (int rr = 0; rr < kFXRows; rr++) {
    long long y = y0 + rr;
    if (y >= H) break;
    const uint32_t* row = in + y * W;
    for (int i = threadIdx.x; i < span; i += kFX) {
      long long gx = x0 - r + i;
      px[rr * span + i] = (gx >= 0 && gx < W) ? px4(row[gx]) : o;
    }
  }
  for (int i = threadIdx.x; i < 2 * r + 1; i += kFX) kw[i] = (float)kern[i];
  __syncthreads();
  const long long x = x0 + threadIdx.x;
  if (x >= W) return;
  for (int rr = 0; rr < kFXRows; rr++) {
    long long y = y0 + rr;
    if (y >= H) break;
    const float4* p = px + rr * span + threadIdx.x;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k <= 2 * r; k++) {
      float4 v = p[k];
      float w = kw[k];
      a.x = fmaf(v.x, w, a.x);
      a.y = fmaf(v.y, w, a.y);
      a.z = fmaf(v.z, w, a.z);
      a.w = fmaf(v.w, w, a.w);
    }
    out[y * W + x] = quantf(a);
  }
}

__global__ void __launch_bounds__(32 * kFYThreads) k_blurf_y(const uint32_t* __restrict__ in,
                                                             uint32_t* __restrict__ out, long long W,
                                                             long long H, int r,
                                                             const uint16_t* __restrict__ kern,
                                                             uint32_t oob) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int span = kFYT + 2 * r;
  float4* px = reinterpret_cast<float4*>(sm);            // span x 32
  float* kw = reinterpret_cast<float*>(px + span * 32);  // 2r + 1
  const long long x0 = (long long)blockIdx.x * 32, y0 = (long long)blockIdx.y * kFYT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long x = x0 + tx;
  const float4 o = px4(oob);
  for (int i = ty; i < span; i += kFYThreads) {
    long long gy = y0 - r + i;
    float4 v = o;
    if (gy >= 0 && gy < H) v = x < W ? px4(in[gy * W + x]) : make_float4(0.f, 0.f, 0.f, 0.f);
    px[i * 32 + tx] = v;
  }
  for (int i = ty * 32 + tx; i < 2 * r + 1; i += 32 * kFYThreads) kw[i] = (float)kern[i];
  __syncthreads();
  if (x >= W) return;
  for (int oy = ty; oy < kFYT; oy += kFYThreads) {
    long long y = y0 + oy;
    if (y >= H) break;
    const float4* p = px + oy * 32 + tx;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k <= 2 * r; k++) {
      float4 v = p[k * 32];
      float w = kw[k];
      a.x = fmaf(v.x, w, a.x);
      a.y = fmaf(v.y, w, a.y);
      a.z = fmaf(v.z, w, a.z);
      a.w = fmaf(v.w, w, a.w);
    }
    out[y * W + x] = quantf(a);
  }
}

size_t blurf_x_smem(int r) { return (size_t)kFXRows * (kFX + 2 * r) * 16 + (size_t)(2 * r + 1) * 4 + 16; }
size_t blurf_y_smem(int r) { return (size_t)(kFYT + 2 * r) * 32 * 16 + (size_t)(2 * r + 1) * 4 + 16; }


// ---- RGBX blur, register-blocked float32 path ---------------------------------
// The tile lives in shared memory as [position along the filter axis][lane],
// where the 32 lanes are 32 rows (X pass) or 32 columns (Y pass), so every
// warp-wide 128-bit load is conflict-free.  Each thread produces 8
// consecutive outputs along the axis from a 16-pixel register window that
// advances 8 taps at a time: 16 shared loads feed 256 FFMAs.
constexpr int kBT = 64;   // outputs along the filter axis per CTA
constexpr int kBP = 8;    // outputs per thread (and taps per block)
constexpr int kBWarps = kBT / kBP;

__host__ __device__ constexpr int blockblur_span(int r) { return kBT + 2 * r + kBP; }
size_t blockblur_smem(int r) {
  return (size_t)blockblur_span(r) * 32 * 16 + (size_t)(2 * r + 1 + kBP) * 4 + 16;
}

template <bool XPASS>
__global__ void __launch_bounds__(kBWarps * 32, 2)
    k_blurb(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, long long W, long long H,
            int r, const uint16_t* __restrict__ kern, uint32_t oob) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int span = blockblur_span(r);
  const int ntap = 2 * r + 1;
  float4* px = reinterpret_cast<float4*>(sm);            // span x 32
  float* kw = reinterpret_cast<float*>(px + span * 32);  // taps, zero-padded to a multiple of 8
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // tile origin: along the axis (a0) and across it (c0)
  const long long a0 = (long long)blockIdx.x * kBT, c0 = (long long)blockIdx.y * 32;
  const long long alen = XPASS ? W : H, clen = XPASS ? H : W;
  const float4 o = px4(oob), zero = make_float4(0.f, 0.f, 0.f, 0.f);
  // Stage the tile: 8 loads per thread in flight before any is converted, so
  // the staging does not wait on L2/HBM latency one pixel at a time.
  constexpr int kU = 8;
  const int total = span * 32;
  for (int i0 = tid; i0 < total; i0 += kU * kBWarps * 32) {
    uint32_t raw[kU];
    int kind[kU];  // 0: zero padding, 1: out of bounds, 2: pixel
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int i = i0 + u * kBWarps * 32;
      int p, c;
      if (XPASS) {  // consecutive threads read consecutive x of one row
        c = i / span;
        p = i - c * span;
      } else {  // consecutive threads read consecutive x of one row
        p = i >> 5;
        c = i & 31;
      }
      const long long ga = a0 - r + p, gc = c0 + c;
      kind[u] = 0;
      raw[u] = 0u;
      if (i < total && p < kBT + 2 * r && gc < clen) {
        if (ga >= 0 && ga < alen) {
          raw[u] = XPASS ? in[gc * W + ga] : in[ga * W + gc];
          kind[u] = 2;
        } else {
          kind[u] = 1;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int i = i0 + u * kBWarps * 32;
      if (i >= total) break;
      int p, c;
      if (XPASS) {
        c = i / span;
        p = i - c * span;
      } else {
        p = i >> 5;
        c = i & 31;
      }
      px[p * 32 + c] = kind[u] == 2 ? px4(raw[u]) : (kind[u] == 1 ? o : zero);
    }
  }
  for (int i = tid; i < ntap + kBP; i += kBWarps * 32) kw[i] = i < ntap ? (float)kern[i] : 0.f;
  __syncthreads();

  const int p0 = warp * kBP;  // this thread's first output along the axis
  float4 acc[kBP];
#pragma unroll
  for (int j = 0; j < kBP; j++) acc[j] = zero;
  for (int kb = 0; kb < ntap; kb += kBP) {
    float4 win[2 * kBP];
#pragma unroll
    for (int i = 0; i < 2 * kBP; i++) win[i] = px[(p0 + kb + i) * 32 + lane];
#pragma unroll
    for (int kk = 0; kk < kBP; kk++) {
      const float w = kw[kb + kk];
#pragma unroll
      for (int j = 0; j < kBP; j++) {
        acc[j].x = fmaf(win[j + kk].x, w, acc[j].x);
        acc[j].y = fmaf(win[j + kk].y, w, acc[j].y);
        acc[j].z = fmaf(win[j + kk].z, w, acc[j].z);
        acc[j].w = fmaf(win[j + kk].w, w, acc[j].w);
      }
    }
  }
  const long long gc = c0 + lane;
  if (XPASS) {
    // stage through shared memory so the row-major stores are coalesced
    __syncthreads();
    uint32_t* st = reinterpret_cast<uint32_t*>(sm);  // 32 rows x kBT
#pragma unroll
    for (int j = 0; j < kBP; j++) st[lane * kBT + p0 + j] = quantf(acc[j]);
    __syncthreads();
    for (int i = tid; i < 32 * kBT; i += kBWarps * 32) {
      int c = i / kBT, p = i - c * kBT;
      long long gy = c0 + c, gx = a0 + p;
      if (gy < H && gx < W) out[gy * W + gx] = st[i];
    }
  } else {
    if (gc < W) {
#pragma unroll
      for (int j = 0; j < kBP; j++) {
        long long gy = a0 + p0 + j;
        if (gy < H) out[gy * W + gc] = quantf(acc[j]);
      }
    }
  }
}

void* blurb_kernel(bool x) { return x ? (void*)k_blurb<true> : (void*)k_blurb<false>; }

// Direct (untiled) passes for radii whose halo does not fit in shared memory.
__global__ void k_blur_x_direct(const uint32_t* in, uint32_t* out, long long W, long long H, int r,
                                const uint16_t* kern, uint32_t oob) {
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long y = i / W, x = i - y * W;
    uint32_t s[4] = {0, 0, 0, 0};
    for (int k = 0; k <= 2 * r; k++) {
      long long gx = x - r + k;
      mac4(s, (gx >= 0 && gx < W) ? in[y * W + gx] : oob, kern[k]);
    }
    out[i] = quant4(s);
  }
}
__global__ void k_blur_y_direct(const uint32_t* in, uint32_t* out, long long W, long long H, int r,
                                const uint16_t* kern, uint32_t oob) {
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long y = i / W, x = i - y * W;
    uint32_t s[4] = {0, 0, 0, 0};
    for (int k = 0; k <= 2 * r; k++) {
      long long gy = y - r + k;
      mac4(s, (gy >= 0 && gy < H) ? in[gy * W + x] : oob, kern[k]);
    }
    out[i] = quant4(s);
  }
}

// ---- alpha-plane passes (shadow) -------------------------------------------
// mask.draw(image, translate(offset), OverwriteBlend), alpha only
__global__ void k_alpha_offset(const uint32_t* src, uint8_t* a, long long W, long long H,
                               long long ox, long long oy) {
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long y = i / W, x = i - y * W;
    long long sx = x - ox, sy = y - oy;
    a[i] = (sx >= 0 && sx < W && sy >= 0 && sy < H) ? (uint8_t)(src[sy * W + sx] >> 24) : 0;
  }
}
// spread: running max (grow) or min (shrink) over [c - s, c + s] clipped to
// the image, along x (dir 0) or y (dir 1)
__global__ void k_spread(const uint8_t* in, uint8_t* out, long long W, long long H, int s, int grow,
                         int dir) {
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long y = i / W, x = i - y * W;
    long long c = dir == 0 ? x : y, len = dir == 0 ? W : H;
    long long lo = c - s < 0 ? 0 : c - s, hi = c + s > len - 1 ? len - 1 : c + s;
    uint32_t v = grow ? 0u : 255u;
    for (long long t = lo; t <= hi; t++) {
      uint32_t p = dir == 0 ? in[y * W + t] : in[t * W + x];
      v = grow ? (p > v ? p : v) : (p < v ? p : v);
    }
    out[i] = (uint8_t)v;
  }
}
__global__ void k_blur_a(const uint8_t* in, uint8_t* out, long long W, long long H, int r,
                         const uint16_t* kern, uint32_t oobA, int dir) {
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long y = i / W, x = i - y * W;
    long long c = dir == 0 ? x : y, len = dir == 0 ? W : H;
    uint32_t s = 0;
    for (int k = 0; k <= 2 * r; k++) {
      long long t = c - r + k;
      uint32_t p = (t >= 0 && t < len) ? (dir == 0 ? in[y * W + t] : in[t * W + x]) : oobA;
      s += p * kern[k];
    }
    out[i] = (uint8_t)(s / 256 / 255);
  }
}
// result.fill(color); result.draw(mask, MaskBlend)  -> color * a / 255
__global__ void k_shadow_out(const uint8_t* a, uint32_t* out, long long n, uint32_t color) {
  Px c = unpack(color);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    uint32_t k = a[i];
    out[i] = pack((c.r * k) / 255, (c.g * k) / 255, (c.b * k) / 255, (c.a * k) / 255);
  }
}
// spread on an RGBX image: writes rgbx(0, 0, 0, v)
__global__ void k_alpha_to_rgbx(const uint8_t* a, uint32_t* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (uint32_t)a[i] << 24;
}
__global__ void k_rgbx_alpha(const uint32_t* in, uint8_t* a, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a[i] = (uint8_t)(in[i] >> 24);
}

static unsigned grid_for(long long n, int nsm) {
  long long b = (n + 255) / 256, cap = (long long)nsm * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

size_t blur_x_smem(int r) { return (size_t)(kBX + 2 * r) * 4 + (size_t)(2 * r + 1) * 2 + 16; }
size_t blur_y_smem(int r) { return (size_t)(kTY + 2 * r) * kTX * 4 + (size_t)(2 * r + 1) * 2 + 16; }

// in -> tmp (X pass) -> in (Y pass); float32 tiles when they fit, then the
// integer tiles, then the direct kernels.


void launch_blur(uint32_t* img, uint32_t* tmp, long long W, long long H, int r,
                 const uint16_t* kern, uint32_t oob, int nsm, size_t maxSmem, cudaStream_t st) {
  // radius >= 8: register-blocked tiles; smaller radii stay on the one-output
  // float32 tiles, where the blocked kernel's 8-tap granularity and halo cost
  // more than they save.
  if (r >= 8 && blockblur_smem(r) <= maxSmem && (H + 31) / 32 <= 65535 && (W + 31) / 32 <= 65535) {
    dim3 gx((unsigned)((W + kBT - 1) / kBT), (unsigned)((H + 31) / 32));
    k_blurb<true><<<gx, kBWarps * 32, blockblur_smem(r), st>>>(img, tmp, W, H, r, kern, oob); note_launch();
    dim3 gy((unsigned)((H + kBT - 1) / kBT), (unsigned)((W + 31) / 32));
    k_blurb<false><<<gy, kBWarps * 32, blockblur_smem(r), st>>>(tmp, img, W, H, r, kern, oob); note_launch();
    return;
  }
  if (blurf_x_smem(r) <= maxSmem && (H + kFXRows - 1) / kFXRows <= 65535) {
    dim3 g((unsigned)((W + kFX - 1) / kFX), (unsigned)((H + kFXRows - 1) / kFXRows));
    k_blurf_x<<<g, kFX, blurf_x_smem(r), st>>>(img, tmp, W, H, r, kern, oob); note_launch();
  } else if (blur_x_smem(r) <= maxSmem && H <= 65535) {
    dim3 g((unsigned)((W + kBX - 1) / kBX), (unsigned)H);
    k_blur_x<<<g, kBX, blur_x_smem(r), st>>>(img, tmp, W, H, r, kern, oob); note_launch();
  } else {
    k_blur_x_direct<<<grid_for(W * H, nsm), 256, 0, st>>>(img, tmp, W, H, r, kern, oob); note_launch();
  }
  if (blurf_y_smem(r) <= maxSmem && (H + kFYT - 1) / kFYT <= 65535) {
    dim3 g((unsigned)((W + 31) / 32), (unsigned)((H + kFYT - 1) / kFYT));
    k_blurf_y<<<g, dim3(32, kFYThreads), blurf_y_smem(r), st>>>(tmp, img, W, H, r, kern, oob); note_launch();
  } else if (blur_y_smem(r) <= maxSmem && (H + kTY - 1) / kTY <= 65535) {
    dim3 g((unsigned)((W + kTX - 1) / kTX), (unsigned)((H + kTY - 1) / kTY));
    k_blur_y<<<g, dim3(kTX, kYThreadsY), blur_y_smem(r), st>>>(tmp, img, W, H, r, kern, oob); note_launch();
  } else {
    k_blur_y_direct<<<grid_for(W * H, nsm), 256, 0, st>>>(tmp, img, W, H, r, kern, oob); note_launch();
  }
}

void launch_spread(uint32_t* img, uint8_t* a0, uint8_t* a1, long long W, long long H, int s,
                   int nsm, cudaStream_t st) {
  long long n = W * H;
  int grow = s > 0, m = s > 0 ? s : -s;
  k_rgbx_alpha<<<grid_for(n, nsm), 256, 0, st>>>(img, a0, n); note_launch();
  k_spread<<<grid_for(n, nsm), 256, 0, st>>>(a0, a1, W, H, m, grow, 0); note_launch();
  k_spread<<<grid_for(n, nsm), 256, 0, st>>>(a1, a0, W, H, m, grow, 1); note_launch();
  k_alpha_to_rgbx<<<grid_for(n, nsm), 256, 0, st>>>(a0, img, n); note_launch();
}

// shadow in one pass over 64 x 64 output tiles: the tile and a halo of
// |spread| + radius (at most kShadowHalo) of the offset alpha plane are staged
// in shared memory and the reference's stages run there in order -- spread
// along x then y (a running max or min over the window clipped to the image:
// positions outside the image hold the neutral value), blur along x then y
// (taps outside the image read 0; integer sums and v div 256 div 255 as the
// blur passes), then colour * alpha / 255 (the MaskBlend draw of the filled
// result) written once.
// The blur radius R is a template parameter (0..kShadowHalo): the taps unroll
// and each thread forms four neighbouring outputs from one window of inputs.
constexpr int kShadowTile = 64, kShadowHalo = 32;
template <int R>
__global__ void __launch_bounds__(1024) k_shadow_tile(const uint32_t* __restrict__ src, uint32_t* __restrict__ out,
                                                     int W, int H, int ox, int oy, int m, int grow,
                                                     const uint16_t* __restrict__ kern, uint32_t color, int late) {
  constexpr int r = R;
  extern __shared__ __align__(16) unsigned char sh[];
  const int h = m + r, S = kShadowTile + 2 * h;  // staged side
  unsigned char* b0 = sh;
  unsigned char* b1 = sh + S * S;
  uint32_t* wk = reinterpret_cast<uint32_t*>(sh + ((2 * S * S + 15) & ~15));
  const int gx0 = blockIdx.x * kShadowTile - h, gy0 = blockIdx.y * kShadowTile - h;  // staged [0][0]
  const int tid = threadIdx.x, T = blockDim.x;
  pdl_late_entry(late);
  if (r > 0)  // without a blur there is no weight table
    for (int k = tid; k <= 2 * r; k += T) wk[k] = kern[k];
  const unsigned char neutral = (m > 0 && !grow) ? 255 : 0;
  auto inside = [&](int i, int j) {
    const int gx = gx0 + j, gy = gy0 + i;
    return gx >= 0 && gx < W && gy >= 0 && gy < H;
  };
  // each warp takes rows, its lanes consecutive columns (no divisions by S)
  const int nw = T >> 5, wi = tid >> 5, ln = tid & 31;
  // the offset alpha plane (k_alpha_offset), neutral outside the image
  for (int i = wi; i < S; i += nw)
    for (int j = ln; j < S; j += 32) {
      const int gx = gx0 + j, gy = gy0 + i;
      unsigned char v = neutral;
      if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
        const int sx = gx - ox, sy = gy - oy;
        v = (sx >= 0 && sx < W && sy >= 0 && sy < H) ? (unsigned char)(src[(long long)sy * W + sx] >> 24) : 0;
      }
      b0[i * S + j] = v;
    }
  __syncthreads();
  if (m > 0) {  // spread along x into b1, then along y back into b0 (rows and columns [m, S - m))
    for (int i = wi; i < S; i += nw)
      for (int j = m + ln; j < S - m; j += 32) {
        const unsigned char* p = b0 + i * S + j - m;
        uint32_t v = neutral;
        if (grow)
          for (int t = 0; t <= 2 * m; t++) v = max(v, (uint32_t)p[t]);
        else
          for (int t = 0; t <= 2 * m; t++) v = min(v, (uint32_t)p[t]);
        b1[i * S + j] = (unsigned char)v;
      }
    __syncthreads();
    for (int i = m + wi; i < S - m; i += nw)
      for (int j = m + ln; j < S - m; j += 32) {
        const unsigned char* p = b1 + (i - m) * S + j;
        uint32_t v = neutral;
        if (grow)
          for (int t = 0; t <= 2 * m; t++) v = max(v, (uint32_t)p[t * S]);
        else
          for (int t = 0; t <= 2 * m; t++) v = min(v, (uint32_t)p[t * S]);
        b0[i * S + j] = inside(i, j) ? (unsigned char)v : 0;  // blur taps outside the image read 0
      }
    __syncthreads();
  } else if (neutral != 0) {
    for (int i = wi; i < S; i += nw)
      for (int j = ln; j < S; j += 32)
        if (!inside(i, j)) b0[i * S + j] = 0;
    __syncthreads();
  }
  const unsigned char* fin = b0;  // final alpha at [h + y][h + x]
  if (r > 0) {
    // blur along x: rows [m, S - m), the tile's columns, into b1 (0 outside the
    // image); a task is four neighbouring outputs of a row
    constexpr int NT = 2 * R + 4;
    for (int task = tid; task < (S - 2 * m) * (kShadowTile / 4); task += T) {
      const int i = m + task / (kShadowTile / 4), j = h + 4 * (task % (kShadowTile / 4));
      const unsigned char* p = b0 + i * S + j - r;
      uint32_t a[4] = {0, 0, 0, 0};
#pragma unroll
      for (int t = 0; t < NT; t++) {
        const uint32_t v = p[t];
#pragma unroll
        for (int o = 0; o < 4; o++)
          if (t - o >= 0 && t - o <= 2 * R) a[o] += v * wk[t - o];
      }
#pragma unroll
      for (int o = 0; o < 4; o++) b1[i * S + j + o] = inside(i, j + o) ? (unsigned char)(a[o] / 256 / 255) : 0;
    }
    __syncthreads();
    // blur along y: the tile, into b0; a task is four neighbouring outputs of a column
    for (int task = tid; task < kShadowTile * (kShadowTile / 4); task += T) {
      const int j = h + task % kShadowTile, i = h + 4 * (task / kShadowTile);
      const unsigned char* p = b1 + (i - r) * S + j;
      uint32_t a[4] = {0, 0, 0, 0};
#pragma unroll
      for (int t = 0; t < NT; t++) {
        const uint32_t v = p[t * S];
#pragma unroll
        for (int o = 0; o < 4; o++)
          if (t - o >= 0 && t - o <= 2 * R) a[o] += v * wk[t - o];
      }
#pragma unroll
      for (int o = 0; o < 4; o++) b0[(i + o) * S + j] = (unsigned char)(a[o] / 256 / 255);
    }
    __syncthreads();
  }
  const Px c = unpack(color);
  for (int idx = tid; idx < kShadowTile * kShadowTile; idx += T) {
    const int y = idx / kShadowTile, x = idx % kShadowTile;
    const int gx = gx0 + h + x, gy = gy0 + h + y;
    if (gx >= W || gy >= H) continue;
    const uint32_t k = fin[(h + y) * S + h + x];
    out[(long long)gy * W + gx] = pack((c.r * k) / 255, (c.g * k) / 255, (c.b * k) / 255, (c.a * k) / 255);
  }
  pdl_late_exit(late);
}
typedef void (*ShadowTileKernel)(const uint32_t*, uint32_t*, int, int, int, int, int, int, const uint16_t*, uint32_t,
                                 int);
template <int R>
struct ShadowTable {
  static void fill(ShadowTileKernel* t) {
    t[R] = k_shadow_tile<R>;
    ShadowTable<R + 1>::fill(t);
  }
};
template <>
struct ShadowTable<kShadowHalo + 1> {
  static void fill(ShadowTileKernel*) {}
};
ShadowTileKernel shadow_tile_kernel(int r) {
  static ShadowTileKernel table[kShadowHalo + 1] = {nullptr};
  if (!table[0]) ShadowTable<0>::fill(table);
  return table[r];
}
size_t shadow_tile_smem(int h) {
  const int S = kShadowTile + 2 * h;
  return (size_t)((2 * S * S + 15) & ~15) + (size_t)(2 * kShadowHalo + 1) * 4;
}

void launch_shadow(const uint32_t* src, uint32_t* out, uint8_t* a0, uint8_t* a1, long long W,
                   long long H, long long ox, long long oy, int s, int r, const uint16_t* kern,
                   uint32_t color, int nsm, cudaStream_t st) {
  long long n = W * H;
  const int m = s > 0 ? s : -s;
  if (m + r <= kShadowHalo && W <= (1 << 24) && H <= (1 << 24) && ox > -(1 << 24) && ox < (1 << 24) &&
      oy > -(1 << 24) && oy < (1 << 24)) {
    const dim3 g((unsigned)((W + kShadowTile - 1) / kShadowTile), (unsigned)((H + kShadowTile - 1) / kShadowTile));
    const int late = dep_late(st, {Span{out, (size_t)(n * 4)}}, {Span{src, (size_t)(n * 4)}});
    launch_pdl(shadow_tile_kernel(r), g, dim3(1024), shadow_tile_smem(m + r), st, src, out, (int)W, (int)H, (int)ox,
               (int)oy, m, (int)(s > 0), kern, color, late);
    note_launch();
    return;
  }
  k_alpha_offset<<<grid_for(n, nsm), 256, 0, st>>>(src, a0, W, H, ox, oy); note_launch();
  if (s != 0) {
    int grow = s > 0, m = s > 0 ? s : -s;
    k_spread<<<grid_for(n, nsm), 256, 0, st>>>(a0, a1, W, H, m, grow, 0); note_launch();
    k_spread<<<grid_for(n, nsm), 256, 0, st>>>(a1, a0, W, H, m, grow, 1); note_launch();
  }
  if (r != 0) {
    k_blur_a<<<grid_for(n, nsm), 256, 0, st>>>(a0, a1, W, H, r, kern, 0u, 0); note_launch();
    k_blur_a<<<grid_for(n, nsm), 256, 0, st>>>(a1, a0, W, H, r, kern, 0u, 1); note_launch();
  }
  k_shadow_out<<<grid_for(n, nsm), 256, 0, st>>>(a0, out, n, color); note_launch();
}

}  // namespace pxg
