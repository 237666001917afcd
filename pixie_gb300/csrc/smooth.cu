// draw with a Mat3 transform (src/pixie/images.nim:636-678): the minifyBy2 /
// magnifyBy2 pre-passes (:168-259) and drawSmooth (:531-634) with bilinear
// sampling by getRgbaSmooth (:367-403) and `mix` (common.nim:59-65).
//
// k_minify2 / k_magnify2 are HBM-bound: one output pixel per thread (minify,
// four 4-byte loads of the 2x2 block), one source pixel per thread (magnify,
// two 8-byte stores of its 2x2 block: both rows start at an even pixel offset,
// 2y * 2w and (2y + 1) * 2w).
//
// drawSmooth in two passes.  The reference walks the sample position along a
// row by repeated addition (srcPos += dx), a sum that is sequential in
// float32.  k_smooth_rows gives each row one thread: it intersects the row's
// two scanlines with the four perimeter segments in the reference's order
// (the row's x span) and runs the row's walk with packed f32x2 adds (IEEE,
// both coordinates at once), storing every 8th position, so a warp
// instruction advances 32 rows.  k_draw_smooth then gives each warp 256 pixels
// of a row; a lane resumes the walk from its stored position for 8 pixels,
// samples each (four gathers, two or three byte-wise mixes) and blends it into
// the destination with the mode's blender.  The positions are the reference's
// floats exactly.
#include <cstdint>

#include "pxg_device.cuh"

namespace pxg {

void note_launch();

namespace {

// floor(v / 255) of both 16-bit lanes, each v <= 65152: (v + 1 + (v >> 8)) >> 8
// (exact for every v < 65536, checked exhaustively; no carry crosses lanes)
__device__ __forceinline__ uint32_t div255x2(uint32_t w) {
  return ((w + 0x00010001u + ((w >> 8) & 0x00FF00FFu)) >> 8) & 0x00FF00FFu;
}
// `mix`(ColorRGBX, ColorRGBX, float32)  common.nim:59-65: per channel
// (a (255 - x) + b x + 127) div 255 with x = round(t * 255) <= 255, two
// channels per 32-bit word (each lane <= 255 * 255 + 127 = 65152)
__device__ __forceinline__ uint32_t mix_px(uint32_t a, uint32_t b, float t) {
  const uint32_t x = nim_u32(roundf(t * 255.0f));
  const uint32_t lo = (a & 0x00FF00FFu) * (255 - x) + (b & 0x00FF00FFu) * x + 0x007F007Fu;
  const uint32_t hi = ((a >> 8) & 0x00FF00FFu) * (255 - x) + ((b >> 8) & 0x00FF00FFu) * x + 0x007F007Fu;
  return div255x2(lo) | (div255x2(hi) << 8);
}
// mix(a, b, 0.5): round(0.5 * 255) = round(127.5) = 128 (half away from zero)
__device__ __forceinline__ uint32_t mix_half(uint32_t a, uint32_t b) {
  const Px p = unpack(a), q = unpack(b);
  return pack((p.r * 127 + q.r * 128 + 127) / 255, (p.g * 127 + q.g * 128 + 127) / 255,
              (p.b * 127 + q.b * 128 + 127) / 255, (p.a * 127 + q.a * 128 + 127) / 255);
}
// c * opacity for opacity 0.5 (x = 128) and 0.25 (x = round(63.75) = 64)
__device__ __forceinline__ uint32_t mul_x(uint32_t c, uint32_t x) {
  const Px p = unpack(c);
  return pack((p.r * x + 127) / 255, (p.g * x + 127) / 255, (p.b * x + 127) / 255, (p.a * x + 127) / 255);
}

// minifyBy2 with power 1: out is ((w + 1) / 2) x ((h + 1) / 2)
__global__ void __launch_bounds__(256) k_minify2(const uint32_t* __restrict__ src, long long w, long long h,
                                                 uint32_t* __restrict__ out) {
  const long long ew = w / 2, eh = h / 2, rw = (w + 1) / 2, rh = (h + 1) / 2;
  const long long n = rw * rh;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long y = i / rw, x = i - y * rw;
    uint32_t v;
    if (x < ew && y < eh) {  // 4-byte loads: an odd width leaves the bottom row's pairs 4-byte aligned only
      const uint32_t* t = src + 2 * y * w + 2 * x;
      const uint32_t* u = t + w;
      const Px a = unpack(t[0]), bb = unpack(t[1]), c = unpack(u[1]), d = unpack(u[0]);
      v = pack((a.r + bb.r + c.r + d.r + 2) / 4, (a.g + bb.g + c.g + d.g + 2) / 4,
               (a.b + bb.b + c.b + d.b + 2) / 4, (a.a + bb.a + c.a + d.a + 2) / 4);
    } else if (y < eh) {  // odd width: the last column  images.nim:201-207
      v = mul_x(mix_half(src[2 * y * w + w - 1], src[(2 * y + 1) * w + w - 1]), 128);
    } else if (x < ew) {  // odd height: the last row  :209-216
      v = mul_x(mix_half(src[(h - 1) * w + 2 * x], src[(h - 1) * w + 2 * x + 1]), 128);
    } else {              // both odd: the corner  :218-220
      v = mul_x(src[(h - 1) * w + w - 1], 64);
    }
    out[i] = v;
  }
}

// magnifyBy2 with power 1: out is 2w x 2h
__global__ void __launch_bounds__(256) k_magnify2(const uint32_t* __restrict__ src, long long w, long long h,
                                                  uint32_t* __restrict__ out) {
  const long long n = w * h;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long y = i / w, x = i - y * w;
    const uint32_t v = src[i];
    const uint2 vv = make_uint2(v, v);
    *reinterpret_cast<uint2*>(out + 2 * y * (2 * w) + 2 * x) = vv;
    *reinterpret_cast<uint2*>(out + (2 * y + 1) * (2 * w) + 2 * x) = vv;
  }
}

}  // namespace

// Geometry of one drawSmooth: p, dx, dy of the inverse transform, the four
// perimeter segments (at.x, at.y, to.x, to.y) and the row range.
struct SmoothArgs {
  float px, py, dxx, dxy, dyx, dyy;
  float seg[4][4];
  long long yStart, yEnd;
};

namespace {

// bumpy intersects(Line, Segment): the segment's parameter t in [0, 1], the
// point taken on the segment (the same form as the band clipping's)
__device__ __forceinline__ bool scan_hit(const float* s, float ly, float& ax, float& ay) {
  const float s1x = s[2] - s[0], s1y = s[3] - s[1];
  const float s2x = 1000.0f - -1000.0f, s2y = ly - ly;
  const float den = (-s2x * s1y + s1x * s2y);
  const float t = (s2x * (s[1] - ly) - s2y * (s[0] - -1000.0f)) / den;
  if (t >= 0 && t <= 1) {
    ax = s[0] + s1x * t;
    ay = s[1] + s1y * t;
    return true;
  }
  return false;
}

// image[x, y]: transparent outside  images.nim:37-40
__device__ __forceinline__ uint32_t px_at(const uint32_t* __restrict__ b, long long bw, long long bh, long long x,
                                          long long y) {
  return (x >= 0 && x < bw && y >= 0 && y < bh) ? __ldg(b + y * bw + x) : 0u;
}

// getRgbaSmooth (not wrapped)  images.nim:367-403
__device__ __forceinline__ uint32_t sample_smooth(const uint32_t* __restrict__ b, long long bw, long long bh, float x,
                                                  float y) {
  const float fx = floorf(x), fy = floorf(y);
  const long long x0 = nim_int(fx), y0 = nim_int(fy);
  const long long x1 = x0 == 9223372036854775807LL ? x0 : x0 + 1, y1 = y0 == 9223372036854775807LL ? y0 : y0 + 1;
  const float xf = x - fx, yf = y - fy;
  if (x0 < -1 || x0 >= bw || y0 < -1 || y0 >= bh) return 0u;  // all four taps outside: transparent
  const uint32_t x0y0 = px_at(b, bw, bh, x0, y0), x1y0 = px_at(b, bw, bh, x1, y0);
  const uint32_t x0y1 = px_at(b, bw, bh, x0, y1), x1y1 = px_at(b, bw, bh, x1, y1);
  uint32_t top = x0y0;
  if (xf > 0 && x0y0 != x1y0) top = mix_px(x0y0, x1y0, xf);
  uint32_t bottom = x0y1;
  if (xf > 0 && x0y1 != x1y1) bottom = mix_px(x0y1, x1y1, xf);
  if (yf != 0 && top != bottom) return mix_px(top, bottom, yf);
  return top;
}

template <int MODE>
__device__ __forceinline__ uint32_t smooth_blend(const uint8_t* tbl, uint32_t a, uint32_t s) {
  if (MODE == kNormal) return blendNormal(a, s);
  if (MODE == kOverwrite) return s;
  if (MODE == kMask) return blendMaskPx(a, s);
  if (MODE == kColorBurn) return blendBurnDodge<true>(tbl, a, s);
  if (MODE == kColorDodge) return blendBurnDodge<false>(tbl, a, s);
  if (MODE == kSoftLight || MODE == kHue || MODE == kSaturation || MODE == kColor || MODE == kLuminosity)
    return blendFloatT<MODE>(tbl, a, s);
  return blend_px(MODE, tbl, a, s);
}

__device__ __forceinline__ uint64_t f2(float x, float y) {
  return ((uint64_t)__float_as_uint(y) << 32) | __float_as_uint(x);
}
// both coordinates of srcPos += dx in one packed add (IEEE round-to-nearest per lane)
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ float f2_x(uint64_t v) { return __uint_as_float((uint32_t)v); }
__device__ __forceinline__ float f2_y(uint64_t v) { return __uint_as_float((uint32_t)(v >> 32)); }

constexpr int kPosStep = 8;   // the row pass keeps every 8th sample position
constexpr int kSegPx = 256;   // pixels per warp of the draw pass (32 lanes x 8)

// Pass 1, one thread per row of [yStart, yEnd): the row's x range
// (images.nim:567-582, the hits folded in the reference's order) and the
// sample positions srcPos at xStart, xStart + 8, ... of the sequential walk
// srcPos += dx (:585-589), stored as pos[k * R + row] (R = rows) so that the
// 32 rows of a warp store 256 contiguous bytes.
__global__ void __launch_bounds__(128) k_smooth_rows(SmoothArgs g, long long W, long long R, int2* __restrict__ rng,
                                                     uint64_t* __restrict__ pos) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long y = g.yStart + r;
  if (y >= g.yEnd) return;
  float xMin = (float)W, xMax = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    float ax = 0.0f, ay = 0.0f;
    const float* s = g.seg[k & 3];
    if (scan_hit(s, (float)y + (float)(k >> 2), ax, ay) && !(s[2] == ax && s[3] == ay)) {
      xMin = nmin(xMin, ax);
      xMax = nmax(xMax, ax);
    }
  }
  long long xStart = nim_int(floorf(xMin)), xEnd = nim_int(ceilf(xMax));
  xStart = xStart < 0 ? 0 : (xStart > W ? W : xStart);
  xEnd = xEnd < 0 ? 0 : (xEnd > W ? W : xEnd);
  rng[r] = make_int2((int)xStart, (int)xEnd);
  float cx = (g.px + g.dxx * (float)xStart) + g.dyx * (float)y;
  float cy = (g.py + g.dxy * (float)xStart) + g.dyy * (float)y;
  uint64_t c = f2(cx - 0.5f, cy - 0.5f);
  const uint64_t d = f2(g.dxx, g.dxy);
  uint64_t* out = pos + r;
  for (long long i = 0; i < xEnd - xStart; i += kPosStep, out += R) {
    *out = c;
#pragma unroll
    for (int u = 0; u < kPosStep; u++) c = f2_add(c, d);
  }
}

// Pass 2: warp (row, segment) handles pixels [256 s, 256 s + 256) of the
// row's span [xStart, xEnd).  Lane j resumes the walk srcPos += dx from the
// stored position of span pixel 256 s + 8 j for 8 pixels, into shared
// memory; the warp then samples and blends 32 consecutive pixels at a time.
// MaskBlend: the warp also clears the part of pixels [256 s, 256 s + 256) of
// the row outside the span (the whole row when the span is empty or the row
// lies outside [yStart, yEnd)).
template <int MODE>
__global__ void __launch_bounds__(256) k_draw_smooth(uint32_t* __restrict__ a, long long W, long long H,
                                                     const uint32_t* __restrict__ b, long long bw, long long bh,
                                                     SmoothArgs g, const int2* __restrict__ rng,
                                                     const uint64_t* __restrict__ pos, long long R, long long rowLo,
                                                     long long rowHi, long long segs, const uint8_t* tbl) {
  // lane j's 8 positions at [9 j, 9 j + 8): the stride of 9 entries keeps the
  // 8-byte stores of each half-warp on distinct bank pairs
  __shared__ uint64_t s_pos[8][32 * 9];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint64_t* sp = s_pos[wib];
  const long long items = (rowHi - rowLo) * segs;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const uint64_t d = f2(g.dxx, g.dxy);
  for (long long it = (long long)blockIdx.x * (blockDim.x >> 5) + wib; it < items; it += warps) {
    const long long y = rowLo + it / segs, sg = it - (it / segs) * segs;
    uint32_t* line = a + y * W;
    const long long s0 = sg * kSegPx;
    if (y < g.yStart || y >= g.yEnd) {  // MaskBlend only: rows the image does not reach
      for (long long x = s0 + lane; x < s0 + kSegPx && x < W; x += 32) line[x] = 0u;
      continue;
    }
    const int2 rr = rng[y - g.yStart];
    const long long xStart = rr.x, xEnd = rr.y, len = xEnd - xStart;
    if (len == 0) continue;  // :583-584
    if (MODE == kMask)       // :612-620: clear [0, xStart) and [xEnd, W)
      for (long long x = s0 + lane; x < s0 + kSegPx && x < W; x += 32)
        if (x < xStart || x >= xEnd) line[x] = 0u;
    if (s0 >= len) continue;
    const long long i0 = s0 + (long long)lane * kPosStep;  // span offset of this lane's 8 positions
    __syncwarp();
    if (i0 < len) {
      uint64_t c = pos[(i0 / kPosStep) * R + (y - g.yStart)];
#pragma unroll
      for (int u = 0; u < kPosStep; u++) {
        sp[lane * 9 + u] = c;
        c = f2_add(c, d);
      }
    }
    __syncwarp();
    const long long n = len - s0 < kSegPx ? len - s0 : kSegPx;
    for (int k = lane; k < n; k += 32) {
      const uint64_t c = sp[(k >> 3) * 9 + (k & 7)];
      const long long x = xStart + s0 + k;
      const uint32_t sv = sample_smooth(b, bw, bh, f2_x(c), f2_y(c));
      line[x] = smooth_blend<MODE>(tbl, line[x], sv);
    }
  }
}

typedef void (*SmoothKernel)(uint32_t*, long long, long long, const uint32_t*, long long, long long, SmoothArgs,
                             const int2*, const uint64_t*, long long, long long, long long, long long,
                             const uint8_t*);
template <int M>
struct SmoothTable {
  static void fill(SmoothKernel* t) {
    t[M] = k_draw_smooth<M>;
    SmoothTable<M + 1>::fill(t);
  }
};
template <>
struct SmoothTable<kNumBlends> {
  static void fill(SmoothKernel*) {}
};

unsigned grid_for(long long items, long long per_block, int nsm) {
  long long blocks = (items + per_block - 1) / per_block;
  const long long cap = (long long)nsm * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (unsigned)blocks;
}

}  // namespace

void launch_minify2(const uint32_t* src, long long w, long long h, uint32_t* out, int nsm, cudaStream_t st) {
  const long long n = ((w + 1) / 2) * ((h + 1) / 2);
  k_minify2<<<grid_for(n, 256, nsm), 256, 0, st>>>(src, w, h, out);
  note_launch();
}

void launch_magnify2(const uint32_t* src, long long w, long long h, uint32_t* out, int nsm, cudaStream_t st) {
  k_magnify2<<<grid_for(w * h, 256, nsm), 256, 0, st>>>(src, w, h, out);
  note_launch();
}

// Scratch of one drawSmooth: per row of [yStart, yEnd) its span (int2) and
// the sample position of every 8th pixel of the span.
long long smooth_scratch_bytes(long long W, long long rows) {
  const long long P = (W + kPosStep - 1) / kPosStep + 1;
  return rows * 8 + rows * P * 8;
}

void launch_draw_smooth(uint32_t* a, long long W, long long H, const uint32_t* b, long long bw, long long bh,
                        const SmoothArgs& g, int mode, const uint8_t* tbl, void* scratch, int nsm,
                        cudaStream_t st) {
  static SmoothKernel table[kNumBlends] = {nullptr};
  if (!table[0]) SmoothTable<0>::fill(table);
  const long long rows = g.yEnd - g.yStart;
  int2* rng = reinterpret_cast<int2*>(scratch);
  uint64_t* pos = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(scratch) + rows * 8);
  if (rows > 0) {
    k_smooth_rows<<<(unsigned)((rows + 127) / 128), 128, 0, st>>>(g, W, rows, rng, pos);
    note_launch();
  }
  const long long lo = mode == kMask ? 0 : g.yStart, hi = mode == kMask ? H : g.yEnd;
  if (hi <= lo) return;
  const long long segs = (W + kSegPx - 1) / kSegPx;
  long long blocks = ((hi - lo) * segs + 7) / 8;
  const long long cap = (long long)nsm * 64;
  if (blocks > cap) blocks = cap;
  table[mode]<<<(unsigned)blocks, 256, 0, st>>>(a, W, H, b, bw, bh, g, rng, pos, rows, lo, hi, segs, tbl);
  note_launch();
}

}  // namespace pxg
