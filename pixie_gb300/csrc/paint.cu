// Non-solid paints (src/pixie/paints.nim): gradient fills, applyOpacity
// (images.nim:261-277) and drawTiled / drawCorrect (images.nim:405-445,
// :680-683), the device parts of fillPath / strokePath with a paint
// (paths.nim:2115-2142, :2178-2210).
//
// All three are one pixel per thread, HBM-bound apart from the angular
// gradient's float-float arctangent.  Every float32 expression keeps the
// reference's operation order (the file is built with -fmad=false).
#include <cfloat>
#include <cstdint>
#include <stdexcept>

#include "paint.cuh"
#include "pxg_device.cuh"

namespace pxg {

void note_launch();

namespace {

constexpr double kPI64 = 3.141592653589793;


// float-float ("double-float") arithmetic: a value is hi + lo with |lo| <=
// ulp(hi) / 2; two_sum and the fused-multiply-add two_prod give exact error
// terms (Dekker, Knuth), so every operation is a fixed sequence of IEEE
// float32 operations.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF quick_two_sum(float a, float b) {
  const float s = a + b;
  return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF two_prod(float a, float b) {
  const float p = a * b;
  return DF{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  DF s = two_sum(x.hi, y.hi);
  const DF t = two_sum(x.lo, y.lo);
  s.lo = s.lo + t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ DF df_neg(DF x) { return DF{-x.hi, -x.lo}; }
__device__ __forceinline__ DF df_mul(DF x, DF y) {
  DF p = two_prod(x.hi, y.hi);
  p.lo = p.lo + (x.hi * y.lo + x.lo * y.hi);
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ DF df_div(DF x, DF y) {
  const float q1 = x.hi / y.hi;
  DF r = df_add(x, df_neg(df_mul(y, DF{q1, 0.0f})));
  const float q2 = r.hi / y.hi;
  r = df_add(r, df_neg(df_mul(y, DF{q2, 0.0f})));
  const float q3 = r.hi / y.hi;
  return df_add(quick_two_sum(q1, q2), DF{q3, 0.0f});
}
__device__ __forceinline__ DF df_sqrt(DF a) {  // a > 0
  const float s = sqrtf(a.hi);
  const DF e = df_add(a, df_neg(two_prod(s, s)));
  return quick_two_sum(s, e.hi / (2.0f * s));
}
#define DF_CONST(v) DF{(float)(v), (float)((v) - (double)(float)(v))}
// atan(x) for x >= 0: pi/2 - atan(1/x) above 1, two halvings
// atan(x) = 2 atan(x / (1 + sqrt(1 + x^2))) to x < 0.2, then 14 Taylor
// terms in Horner form
__device__ __forceinline__ DF df_atan_unit(DF x) {
  const DF one{1.0f, 0.0f};
  const bool inv = x.hi > 1.0f || (x.hi == 1.0f && x.lo > 0.0f);
  if (inv) x = df_div(one, x);
  x = df_div(x, df_add(one, df_sqrt(df_add(one, df_mul(x, x)))));
  x = df_div(x, df_add(one, df_sqrt(df_add(one, df_mul(x, x)))));
  const DF x2 = df_mul(x, x);
  DF poly = DF_CONST(-1.0 / 27);
  poly = df_add(df_mul(poly, x2), DF_CONST(1.0 / 25));
  poly = df_add(df_mul(poly, x2), DF_CONST(-1.0 / 23));
  poly = df_add(df_mul(poly, x2), DF_CONST(1.0 / 21));
  poly = df_add(df_mul(poly, x2), DF_CONST(-1.0 / 19));
  poly = df_add(df_mul(poly, x2), DF_CONST(1.0 / 17));
  poly = df_add(df_mul(poly, x2), DF_CONST(-1.0 / 15));
  poly = df_add(df_mul(poly, x2), DF_CONST(1.0 / 13));
  poly = df_add(df_mul(poly, x2), DF_CONST(-1.0 / 11));
  poly = df_add(df_mul(poly, x2), DF_CONST(1.0 / 9));
  poly = df_add(df_mul(poly, x2), DF_CONST(-1.0 / 7));
  poly = df_add(df_mul(poly, x2), DF_CONST(1.0 / 5));
  poly = df_add(df_mul(poly, x2), DF_CONST(-1.0 / 3));
  poly = df_add(df_mul(poly, x2), one);
  const DF sum = df_mul(df_mul(x, poly), DF{4.0f, 0.0f});
  return inv ? df_add(DF_CONST(1.5707963267948966), df_neg(sum)) : sum;
}
// atan2 of float32 arguments rounded to float32 (correctly rounded but for
// true values within ~2^-40 of a rounding boundary)
__device__ __forceinline__ float atan2_cr(float y, float x) {
  if (isnan(x) || isnan(y)) return __int_as_float(0x7fc00000);
  DF r;
  if (y == 0) {
    r = signbit(x) ? DF_CONST(3.141592653589793) : DF{0.0f, 0.0f};
  } else if (x == 0) {
    r = DF_CONST(1.5707963267948966);
  } else if (isinf(x) || isinf(y)) {
    if (isinf(x) && isinf(y))
      r = x > 0 ? DF_CONST(0.7853981633974483) : DF_CONST(2.356194490192345);
    else if (isinf(x))
      r = x > 0 ? DF{0.0f, 0.0f} : DF_CONST(3.141592653589793);
    else
      r = DF_CONST(1.5707963267948966);
  } else {
    const DF q = df_div(DF{fabsf(y), 0.0f}, DF{fabsf(x), 0.0f});
    const DF a = df_atan_unit(q);
    r = x > 0 ? a : df_add(DF_CONST(3.141592653589793), df_neg(a));
  }
  const float v = r.hi + r.lo;
  return signbit(y) ? -v : v;
}

// fixAngle: a float32 compared with the float64 PI, stepped by float32 tau
__device__ __forceinline__ float fix_angle(float a) {
  const float tau = (float)(kPI64 * 2);
  while ((double)a > kPI64) a -= tau;
  while ((double)a < -kPI64) a += tau;
  return a;
}
__device__ __forceinline__ uint32_t color_rgbx(float r, float g, float b, float a) {  // chroma asRgbx
  return premul8(pack(unit_to_u8(r), unit_to_u8(g), unit_to_u8(b), unit_to_u8(a)));
}

// gradientColor  paints.nim:68-93 (chroma mix: a + (b - a) * t per component)
__device__ uint32_t gradient_color(const float* __restrict__ st, int n, float opacity, float t) {
  int index = -1;
  for (int i = 0; i < n; i++) {
    const float pos = st[5 * i + 4];
    if (pos < t) index = i;
    if (pos > t) break;
  }
  float c[4];
  if (index == -1) {
    for (int k = 0; k < 4; k++) c[k] = st[k];
  } else if (index + 1 >= n) {
    for (int k = 0; k < 4; k++) c[k] = st[5 * index + k];
  } else {
    const float* a = st + 5 * index;
    const float* b = a + 5;
    const float u = (t - a[4]) / (b[4] - a[4]);
    for (int k = 0; k < 4; k++) c[k] = a[k] + (b[k] - a[k]) * u;
  }
  c[3] *= opacity;
  return color_rgbx(c[0], c[1], c[2], c[3]);
}

// STAGED: the stops are copied into shared memory once per CTA; otherwise
// (more stops than 48 KB of shared memory holds) they are read from global
// memory, through the read-only cache.
template <int KIND, bool STAGED>
__global__ void __launch_bounds__(256) k_gradient(uint32_t* __restrict__ img, long long W, long long H, GradientArgs g,
                                                  const float* __restrict__ gstops) {
  extern __shared__ float staged[];
  const float* stops = gstops;
  if (STAGED) {
    for (int i = threadIdx.x; i < 5 * g.nstops; i += blockDim.x) staged[i] = gstops[i];
    __syncthreads();
    stops = staged;
  }
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long y = i / W, x = i - y * W;
    const float fx = (float)x, fy = (float)y;
    float t;
    if (KIND == 3) {  // toLineSpace  paints.nim:111-116
      t = (g.dy * (fy - g.aty) + g.dx * (fx - g.atx)) / g.det;
    } else if (KIND == 4) {  // (mat * xy).length()  :201-203
      const float vx = g.m[0] * fx + g.m[3] * fy + g.m[6], vy = g.m[1] * fx + g.m[4] * fy + g.m[7];
      t = sqrtf(vx * vx + vy * vy);
    } else {  // :222-227
      const float vx = fx - g.cx, vy = fy - g.cy;
      const float len = sqrtf(vx * vx + vy * vy);
      const float angle = atan2_cr(vy / len, vx / len);
      const float f32PI = (float)kPI64;
      t = fix_angle(angle + g.gradientAngle + f32PI / 2) / 2 / f32PI + 0.5f;
    }
    img[i] = gradient_color(stops, g.nstops, g.opacity, t);
  }
}

// applyOpacity with o = round(255 * opacity) in 1..254: (c * o) div 255
__global__ void __launch_bounds__(256) k_apply_opacity(uint32_t* __restrict__ img, long long n, uint32_t o) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const Px p = unpack(img[i]);
    img[i] = pack((p.r * o) / 255, (p.g * o) / 255, (p.b * o) / 255, (p.a * o) / 255);
  }
}

__device__ __forceinline__ uint32_t mix_rgbx(uint32_t a, uint32_t b, float t) {  // common.nim:59-65
  const uint32_t x = nim_u32(roundf(t * 255.0f));
  const Px p = unpack(a), q = unpack(b);
  return pack((p.r * (255 - x) + q.r * x + 127) / 255, (p.g * (255 - x) + q.g * x + 127) / 255,
              (p.b * (255 - x) + q.b * x + 127) / 255, (p.a * (255 - x) + q.a * x + 127) / 255);
}

// getRgbaSmooth, wrapped (images.nim:381-385) when TILED: the taps are
// data[w * (y mod h) + (x mod w)] with Nim's truncating mod, read linearly;
// an address outside the buffer reads transparent.  Not wrapped: image[x, y],
// transparent outside.
template <bool TILED>
__device__ __forceinline__ uint32_t tap(const uint32_t* __restrict__ b, long long bw, long long bh, long long x,
                                        long long y) {
  if (TILED) {
    const long long i = bw * (y % bh) + (x % bw);
    return (i >= 0 && i < bw * bh) ? __ldg(b + i) : 0u;
  }
  return (x >= 0 && x < bw && y >= 0 && y < bh) ? __ldg(b + y * bw + x) : 0u;
}
template <bool TILED>
__device__ uint32_t sample(const uint32_t* __restrict__ b, long long bw, long long bh, float x, float y) {
  const float fx = floorf(x), fy = floorf(y);
  const long long x0 = nim_int(fx), y0 = nim_int(fy);
  const long long x1 = x0 == 9223372036854775807LL ? x0 : x0 + 1, y1 = y0 == 9223372036854775807LL ? y0 : y0 + 1;
  const float xf = x - fx, yf = y - fy;
  const uint32_t x0y0 = tap<TILED>(b, bw, bh, x0, y0), x1y0 = tap<TILED>(b, bw, bh, x1, y0);
  const uint32_t x0y1 = tap<TILED>(b, bw, bh, x0, y1), x1y1 = tap<TILED>(b, bw, bh, x1, y1);
  uint32_t top = x0y0;
  if (xf > 0 && x0y0 != x1y0) top = mix_rgbx(x0y0, x1y0, xf);
  uint32_t bottom = x0y1;
  if (xf > 0 && x0y1 != x1y1) bottom = mix_rgbx(x0y1, x1y1, xf);
  if (yf != 0 && top != bottom) return mix_rgbx(top, bottom, yf);
  return top;
}

template <int MODE>
__device__ __forceinline__ uint32_t blend_mode_px(const uint8_t* tbl, uint32_t a, uint32_t s) {
  if (MODE == kNormal) return blendNormal(a, s);
  if (MODE == kOverwrite) return s;
  if (MODE == kMask) return blendMaskPx(a, s);
  return blend_px(MODE, tbl, a, s);
}

// drawCorrect's per-pixel loop: every destination pixel samples
// inverseTransform * (x + h, y + h) - h and blends
template <int MODE, bool TILED>
__global__ void __launch_bounds__(256) k_draw_correct(uint32_t* __restrict__ a, long long W, long long H,
                                                      const uint32_t* __restrict__ b, long long bw, long long bh,
                                                      Mat9 inv, const uint8_t* tbl) {
  const long long n = W * H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long y = i / W, x = i - y * W;
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    const float sx = inv.m[0] * px + inv.m[3] * py + inv.m[6], sy = inv.m[1] * px + inv.m[4] * py + inv.m[7];
    const uint32_t s = sample<TILED>(b, bw, bh, sx - 0.5f, sy - 0.5f);
    a[i] = blend_mode_px<MODE>(tbl, a[i], s);
  }
}

unsigned grid(long long n, int nsm) {
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  return (unsigned)(blocks < 1 ? 1 : blocks);
}

typedef void (*CorrectKernel)(uint32_t*, long long, long long, const uint32_t*, long long, long long, Mat9,
                              const uint8_t*);
template <int M>
struct CorrectTable {
  static void fill(CorrectKernel* t, CorrectKernel* u) {
    t[M] = k_draw_correct<M, true>;
    u[M] = k_draw_correct<M, false>;
    CorrectTable<M + 1>::fill(t, u);
  }
};
template <>
struct CorrectTable<kNumBlends> {
  static void fill(CorrectKernel*, CorrectKernel*) {}
};

}  // namespace

void launch_gradient(uint32_t* img, long long W, long long H, const GradientArgs& g, const float* stops, int nsm,
                     cudaStream_t st) {
  const long long n = W * H;
  const size_t need = sizeof(float) * 5 * (size_t)g.nstops;
  const bool staged = need <= 48 * 1024;
  const size_t smem = staged ? need : 0;
  long long blocks = (n + 255) / 256;  // four waves of eight CTAs per SM at most
  if (blocks > (long long)nsm * 32) blocks = (long long)nsm * 32;
  const unsigned gb = (unsigned)(blocks < 1 ? 1 : blocks);
  if (g.kind == 3)
    (staged ? k_gradient<3, true> : k_gradient<3, false>)<<<gb, 256, smem, st>>>(img, W, H, g, stops);
  else if (g.kind == 4)
    (staged ? k_gradient<4, true> : k_gradient<4, false>)<<<gb, 256, smem, st>>>(img, W, H, g, stops);
  else
    (staged ? k_gradient<5, true> : k_gradient<5, false>)<<<gb, 256, smem, st>>>(img, W, H, g, stops);
  note_launch();
}

void launch_apply_opacity(uint32_t* img, long long n, uint32_t o, int nsm, cudaStream_t st) {
  k_apply_opacity<<<grid(n, nsm), 256, 0, st>>>(img, n, o);
  note_launch();
}

void launch_draw_correct(uint32_t* a, long long W, long long H, const uint32_t* b, long long bw, long long bh,
                         const Mat9& inv, int mode, bool tiled, const uint8_t* tbl, int nsm, cudaStream_t st) {
  static CorrectKernel tiledK[kNumBlends] = {nullptr}, plainK[kNumBlends] = {nullptr};
  if (!tiledK[0]) CorrectTable<0>::fill(tiledK, plainK);
  (tiled ? tiledK : plainK)[mode]<<<grid(W * H, nsm), 256, 0, st>>>(a, W, H, b, bw, bh, inv, tbl);
  note_launch();
}

}  // namespace pxg
