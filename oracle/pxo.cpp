// ORACLE — test infrastructure only.
//
// A CPU restatement, in plain C++17, of the scalar semantics (the
// `-d:pixieNoSimd` build) of pixie 6.0.0's raster hot path:
//   fill/stroke  src/pixie/paths.nim:654-2175
//   blend modes  src/pixie/blends.nim:15-299
//   colour math  src/pixie/common.nim:59-101, src/pixie/internal.nim:17-98
//   draw / blur / spread / shadow   src/pixie/images.nim:55-57,261-365,447-529,636-678,700-776
// Every function below cites the reference line it follows.  It is the
// checker the CUDA library is compared against: only tests/, the smoke check
// and bench.py's CPU-baseline / reference arm may load it, never the product.
//
// Pinning.  The reference is Nim and cannot be built here (no Nim toolchain;
// vmath/chroma/bumpy/nimsimd are not vendored).  This restatement is pinned
// against the reference's own golden PNGs and known-answer asserts
// (tests/golden/make_fixtures.py copies them into tests/golden/*.npz and
// tests/test_oracle_goldens.py checks them).  Helpers that live in the
// unvendored dependencies are restated from their mathematical definition;
// each one says so where it is defined.  The five chroma float blend modes
// (SoftLight, Hue, Saturation, Color, Luminosity) and the chroma
// un-premultiply used by ColorBurn/ColorDodge have no golden: parity for
// them is UNPINNED (W3C Compositing Level 1 formulas, rounding stated below).
//
// Float semantics.  Nim float32 stays float32: this file is compiled with
// -O2 -ffp-contract=off -fno-fast-math (no FMA contraction, IEEE ops in
// source order).  Nim's float->int conversions are C casts, which are
// undefined out of range; we follow what the reference's CI machines
// (x86-64, where the goldens were produced) do: cvttss2si returns the
// "integer indefinite" value INT_MIN for NaN/out-of-range input.

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "simd_lines.h"

namespace pxo {

struct PixieError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------
// Nim scalar conversions (x86-64 cvtts* semantics)
// ---------------------------------------------------------------------------
static inline int64_t nim_int(float f) {  // float32.int
  if (!(f >= -9223372036854775808.0f && f < 9223372036854775808.0f)) return INT64_MIN;
  return (int64_t)f;
}
static inline int32_t nim_i32(float f) {  // float32.int32 / Fixed32(f)
  if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
  return (int32_t)f;
}
// float32.uint32 / .uint16 / .uint8: gcc lowers these through a 64-bit
// (uint32) or 32-bit (uint16/uint8) truncating convert and keeps the low bits.
static inline uint32_t nim_u32(float f) { return (uint32_t)(uint64_t)nim_int(f); }
static inline uint16_t nim_u16(float f) { return (uint16_t)(uint32_t)nim_i32(f); }
static inline uint8_t nim_u8(float f) { return (uint8_t)(uint32_t)nim_i32(f); }

// Nim's system min/max on floats.
static inline float nmin(float x, float y) { return x <= y ? x : y; }
static inline float nmax(float x, float y) { return y <= x ? x : y; }

static const double kPI = 3.141592653589793;            // Nim's PI (float64)
static const float kEpsilon = (float)(0.0001 * kPI);     // paths.nim:44
static const float kPixelErrorMargin = 0.2f;             // paths.nim:45

// ---------------------------------------------------------------------------
// Colours
// ---------------------------------------------------------------------------
struct RGBX {
  uint8_t r, g, b, a;
};
static inline RGBX rgbx(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
  return RGBX{(uint8_t)r, (uint8_t)g, (uint8_t)b, (uint8_t)a};
}
static inline bool same(RGBX p, RGBX q) {
  return p.r == q.r && p.g == q.g && p.b == q.b && p.a == q.a;
}

// chroma Color -> ColorRGBX (`asRgbx`, paths.nim:1603; images.nim:57).
// chroma is not vendored; restated as: straight float -> 8-bit by
// round(c*255) (half away from zero, clamped), then premultiply with
// (c*a+127) div 255.  Pinned by the known answer
// `color(1.0,0.5,0.25,1.0) -> rgbx(255,128,64,255)` (tests/test_images_draw.nim:282)
// and by the exhaustive rgba->rgbx assert (tests/test_images.nim:204-228).
static inline uint8_t unit_to_u8(float c) {
  float v = roundf(c * 255.0f);
  if (!(v > 0.0f)) return 0;
  if (v > 255.0f) return 255;
  return (uint8_t)v;
}
static inline RGBX premultiply(uint8_t r, uint8_t g, uint8_t b, uint8_t a) {
  // internal.nim:86-96
  if (a == 255) return RGBX{r, g, b, a};
  return rgbx((r * (uint32_t)a + 127) / 255, (g * (uint32_t)a + 127) / 255,
              (b * (uint32_t)a + 127) / 255, a);
}
static inline RGBX color_to_rgbx(const float c[4]) {
  return premultiply(unit_to_u8(c[0]), unit_to_u8(c[1]), unit_to_u8(c[2]), unit_to_u8(c[3]));
}

// `*`(ColorRGBX, float32)  common.nim:67-77
static inline RGBX mul_f(RGBX c, float opacity) {
  if (opacity == 0) return RGBX{0, 0, 0, 0};
  uint32_t x = nim_u32(roundf(opacity * 255.0f));
  return rgbx((c.r * x + 127) / 255, (c.g * x + 127) / 255, (c.b * x + 127) / 255,
              (c.a * x + 127) / 255);
}
// Golden-pinning mode (never the parity oracle).  The reference's master PNGs
// were written by a build that (a) floors the coverage multiply
// `rgbx * coverage` ((c*k) div 255, the rounding of the x86 SIMD loops,
// simd/sse2.nim:510-524) and (b) colours trapezoid slivers with the x86 SSE2
// applyOpacity, round-half-even(c * area) (simd/sse2.nim:6-11).  With these
// two knobs the oracle reproduces every golden exactly; without them it is
// the scalar -d:pixieNoSimd semantics of the current source, which the CUDA
// library must match.
int g_golden_mode = 0;

// `*`(ColorRGBX, uint8)  common.nim:79-90
static inline RGBX mul_c(RGBX c, uint8_t k) {
  if (k == 0) return RGBX{0, 0, 0, 0};
  if (g_golden_mode && k != 255)
    return rgbx((c.r * (uint32_t)k) / 255, (c.g * (uint32_t)k) / 255, (c.b * (uint32_t)k) / 255,
                (c.a * (uint32_t)k) / 255);
  if (k == 255) return c;
  return rgbx((c.r * (uint32_t)k + 127) / 255, (c.g * (uint32_t)k + 127) / 255,
              (c.b * (uint32_t)k + 127) / 255, (c.a * (uint32_t)k + 127) / 255);
}

// straightAlphaTable  internal.nim:68-74.  It is a `const`, so Nim evaluates it
// at compile time in its VM, where float arithmetic is float64 (pinned by the
// goldens: e.g. c=14, a=28 gives 127.5 -> 128, which float32 would round to 127).
static uint8_t g_straight[256][256];
static bool g_straight_init = false;
static void init_straight() {
  if (g_straight_init) return;
  for (int a = 0; a < 256; a++) {
    double mult = a > 0 ? (255.0 / (double)a) : 0.0;
    for (int c = 0; c < 256; c++) {
      double v = round((double)c * mult);
      g_straight[a][c] = (uint8_t)(v < 255.0 ? v : 255.0);
    }
  }
  g_straight_init = true;
}

// ---------------------------------------------------------------------------
// Blend modes  blends.nim
// ---------------------------------------------------------------------------
enum Blend {
  NormalBlend = 0, DarkenBlend, MultiplyBlend, ColorBurnBlend, LightenBlend, ScreenBlend,
  ColorDodgeBlend, OverlayBlend, SoftLightBlend, HardLightBlend, DifferenceBlend,
  ExclusionBlend, HueBlend, SaturationBlend, ColorBlend, LuminosityBlend,
  MaskBlend, OverwriteBlend, SubtractMaskBlend, ExcludeMaskBlend, kNumBlends
};

static inline uint8_t blendAlpha(uint8_t b, uint8_t s) {  // blends.nim:41-43
  return (uint8_t)(s + (uint8_t)((b * (uint32_t)(255 - s)) / 255));
}
static inline uint8_t screen(uint32_t b, uint32_t s) {  // blends.nim:45-46
  return (uint8_t)((int32_t)(b + s) - (int32_t)((b * s) / 255));
}
static inline uint8_t hardLight(uint32_t bc, uint32_t ba, uint32_t sc, uint32_t sa) {  // :48-58
  if (sc * 2 <= sa)
    return (uint8_t)((2 * sc * bc + sc * (255 - ba) + bc * (255 - sa)) / 255);
  return screen(bc, sc);
}

static RGBX blendNormal(RGBX b, RGBX s) {  // blends.nim:60-70
  if (b.a == 0 || s.a == 255) return s;
  if (s.a == 0) return b;
  uint32_t k = 255 - (uint32_t)s.a;
  RGBX r;
  r.r = (uint8_t)(s.r + (uint8_t)((b.r * k) / 255));
  r.g = (uint8_t)(s.g + (uint8_t)((b.g * k) / 255));
  r.b = (uint8_t)(s.b + (uint8_t)((b.b * k) / 255));
  r.a = blendAlpha(b.a, s.a);
  return r;
}
static inline uint8_t darken1(uint8_t bc, uint8_t ba, uint8_t sc, uint8_t sa) {  // :73-79
  uint32_t x = bc + ((uint32_t)(uint8_t)(255 - ba) * sc) / 255;
  uint32_t y = sc + ((uint32_t)(uint8_t)(255 - sa) * bc) / 255;
  return (uint8_t)(x < y ? x : y);
}
static inline uint8_t lighten1(uint8_t bc, uint8_t ba, uint8_t sc, uint8_t sa) {  // :129-135
  uint32_t x = bc + ((uint32_t)(uint8_t)(255 - ba) * sc) / 255;
  uint32_t y = sc + ((uint32_t)(uint8_t)(255 - sa) * bc) / 255;
  return (uint8_t)(x > y ? x : y);
}
static inline uint8_t multiply1(uint8_t bc, uint8_t ba, uint8_t sc, uint8_t sa) {  // :87-95
  return (uint8_t)(((uint32_t)(uint8_t)(255 - ba) * sc + (uint32_t)(uint8_t)(255 - sa) * bc +
                    (uint32_t)bc * sc) / 255);
}
static inline uint8_t difference1(uint8_t bc, uint8_t ba, uint8_t sc, uint8_t sa) {  // :191-198
  // (backdropColor + sourceColor) is uint8 + uint8 in Nim: it wraps.
  uint32_t m1 = (uint32_t)bc * sa, m2 = (uint32_t)sc * ba;
  int32_t mn = (int32_t)((m1 < m2 ? m1 : m2) / 255);
  return (uint8_t)((int32_t)(uint8_t)(bc + sc) - 2 * mn);
}
static inline uint8_t exclusion1(uint32_t b, uint32_t s) {  // :207-209
  int32_t v = (int32_t)(b + s) - (int32_t)((2 * b * s) / 255);
  return (uint8_t)(v > 0 ? v : 0);
}

// chroma ColorRGBX -> ColorRGBA (un-premultiply) used by ColorBurn/ColorDodge
// and by the float modes.  chroma is not vendored; UNPINNED.  Restated with
// pixie's own un-premultiply rule, the straightAlphaTable (internal.nim:68-74).
struct RGBA8 {
  uint8_t r, g, b, a;
};
static inline RGBA8 to_straight(RGBX c) {
  init_straight();
  return RGBA8{g_straight[c.a][c.r], g_straight[c.a][c.g], g_straight[c.a][c.b], c.a};
}

static RGBA8 alphaFix(RGBA8 bd, RGBA8 src, RGBA8 mixed) {  // blends.nim:18-39
  uint32_t sa = src.a, ba = bd.a;
  uint32_t t0 = sa * (255 - ba), t1 = sa * ba, t2 = (255 - sa) * ba;
  uint32_t r = t0 * src.r + t1 * mixed.r + t2 * bd.r;
  uint32_t g = t0 * src.g + t1 * mixed.g + t2 * bd.g;
  uint32_t b = t0 * src.b + t1 * mixed.b + t2 * bd.b;
  uint32_t a = sa + ba * (255 - sa) / 255;
  RGBA8 res{0, 0, 0, 0};
  if (a == 0) return res;
  res.r = (uint8_t)(r / a / 255);
  res.g = (uint8_t)(g / a / 255);
  res.b = (uint8_t)(b / a / 255);
  res.a = (uint8_t)a;
  return res;
}
static inline uint8_t colorBurn1(uint32_t b, uint32_t s) {  // :115-121
  if (b == 255) return 255;
  if (s == 0) return 0;
  uint32_t v = (255 * (255 - b)) / s;
  return (uint8_t)(255 - (uint8_t)(v < 255 ? v : 255));
}
static inline uint8_t colorDodge1(uint32_t b, uint32_t s) {  // :162-168
  if (b == 0) return 0;
  if (s == 255) return 255;
  uint32_t v = (255 * b) / (255 - s);
  return (uint8_t)(v < 255 ? v : 255);
}

// ---- chroma float modes (UNPINNED: W3C Compositing Level 1) --------------
// Colour conversion: premultiplied 8-bit -> straight 8-bit (table above) ->
// float c/255.  Blend B(Cb,Cs) per W3C on straight floats, then the W3C
// general formula with source-over:  Cs' = (1-ab)*Cs + ab*B;
// co = as*Cs' + (1-as)*ab*Cb;  ao = as + ab*(1-as);  straight = co/ao,
// back to 8-bit by round(x*255) clamped, then premultiplied (c*a+127) div 255.
struct F3 {
  float r, g, b;
};
static inline float lum3(F3 c) { return 0.3f * c.r + 0.59f * c.g + 0.11f * c.b; }
static inline F3 clipColor(F3 c) {
  float l = lum3(c);
  float n = fminf(c.r, fminf(c.g, c.b));
  float x = fmaxf(c.r, fmaxf(c.g, c.b));
  if (n < 0.0f) {
    float d = l - n;
    c.r = l + ((c.r - l) * l) / d;
    c.g = l + ((c.g - l) * l) / d;
    c.b = l + ((c.b - l) * l) / d;
  }
  if (x > 1.0f) {
    float d = x - l;
    float k = 1.0f - l;
    c.r = l + ((c.r - l) * k) / d;
    c.g = l + ((c.g - l) * k) / d;
    c.b = l + ((c.b - l) * k) / d;
  }
  return c;
}
static inline F3 setLum(F3 c, float l) {
  float d = l - lum3(c);
  return clipColor(F3{c.r + d, c.g + d, c.b + d});
}
static inline float sat3(F3 c) {
  return fmaxf(c.r, fmaxf(c.g, c.b)) - fminf(c.r, fminf(c.g, c.b));
}
static inline F3 setSat(F3 c, float s) {
  float* v[3] = {&c.r, &c.g, &c.b};
  // order indices by value: mx, md, mn (ties resolved by channel order)
  int imax = 0, imin = 0;
  for (int i = 1; i < 3; i++) {
    if (*v[i] > *v[imax]) imax = i;
    if (*v[i] < *v[imin]) imin = i;
  }
  if (imax == imin) {  // all equal
    return F3{0.0f, 0.0f, 0.0f};
  }
  int imid = 3 - imax - imin;
  float cmax = *v[imax], cmin = *v[imin], cmid = *v[imid];
  float out[3];
  if (cmax > cmin) {
    out[imid] = ((cmid - cmin) * s) / (cmax - cmin);
    out[imax] = s;
  } else {
    out[imid] = 0.0f;
    out[imax] = 0.0f;
  }
  out[imin] = 0.0f;
  return F3{out[0], out[1], out[2]};
}
static inline float softLight1(float cb, float cs) {
  if (cs <= 0.5f) return cb - ((1.0f - 2.0f * cs) * cb) * (1.0f - cb);
  float d = cb <= 0.25f ? ((16.0f * cb - 12.0f) * cb + 4.0f) * cb : sqrtf(cb);
  return cb + (2.0f * cs - 1.0f) * (d - cb);
}
static RGBX blendFloat(RGBX bp, RGBX sp, int mode) {
  RGBA8 b8 = to_straight(bp), s8 = to_straight(sp);
  F3 cb{b8.r / 255.0f, b8.g / 255.0f, b8.b / 255.0f};
  F3 cs{s8.r / 255.0f, s8.g / 255.0f, s8.b / 255.0f};
  float ab = b8.a / 255.0f, as = s8.a / 255.0f;
  F3 m;
  switch (mode) {
    case SoftLightBlend:
      m = F3{softLight1(cb.r, cs.r), softLight1(cb.g, cs.g), softLight1(cb.b, cs.b)};
      break;
    case HueBlend: m = setLum(setSat(cs, sat3(cb)), lum3(cb)); break;
    case SaturationBlend: m = setLum(setSat(cb, sat3(cs)), lum3(cb)); break;
    case ColorBlend: m = setLum(cs, lum3(cb)); break;
    default: m = setLum(cb, lum3(cs)); break;  // LuminosityBlend
  }
  float ao = as + ab * (1.0f - as);
  if (!(ao > 0.0f)) return RGBX{0, 0, 0, 0};
  float k = (1.0f - as) * ab;
  float csr = (1.0f - ab) * cs.r + ab * m.r;
  float csg = (1.0f - ab) * cs.g + ab * m.g;
  float csb = (1.0f - ab) * cs.b + ab * m.b;
  float orr = (as * csr + k * cb.r) / ao;
  float og = (as * csg + k * cb.g) / ao;
  float ob = (as * csb + k * cb.b) / ao;
  return premultiply(unit_to_u8(orr), unit_to_u8(og), unit_to_u8(ob), unit_to_u8(ao));
}

// blender(mode)(backdrop, source)  blends.nim:275-299
static RGBX blend_px(int mode, RGBX b, RGBX s) {
  RGBX r;
  switch (mode) {
    case NormalBlend: return blendNormal(b, s);
    case DarkenBlend:  // :72-84
      r.r = darken1(b.r, b.a, s.r, s.a);
      r.g = darken1(b.g, b.a, s.g, s.a);
      r.b = darken1(b.b, b.a, s.b, s.a);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case MultiplyBlend:  // :86-100
      r.r = multiply1(b.r, b.a, s.r, s.a);
      r.g = multiply1(b.g, b.a, s.g, s.a);
      r.b = multiply1(b.b, b.a, s.b, s.a);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case ColorBurnBlend: {  // :111-126
      RGBA8 bd = to_straight(b), sr = to_straight(s), m;
      m.r = colorBurn1(bd.r, sr.r);
      m.g = colorBurn1(bd.g, sr.g);
      m.b = colorBurn1(bd.b, sr.b);
      m.a = 0;
      RGBA8 f = alphaFix(bd, sr, m);
      return premultiply(f.r, f.g, f.b, f.a);
    }
    case LightenBlend:  // :128-140
      r.r = lighten1(b.r, b.a, s.r, s.a);
      r.g = lighten1(b.g, b.a, s.g, s.a);
      r.b = lighten1(b.b, b.a, s.b, s.a);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case ScreenBlend:  // :142-146
      r.r = screen(b.r, s.r);
      r.g = screen(b.g, s.g);
      r.b = screen(b.b, s.b);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case ColorDodgeBlend: {  // :158-173
      RGBA8 bd = to_straight(b), sr = to_straight(s), m;
      m.r = colorDodge1(bd.r, sr.r);
      m.g = colorDodge1(bd.g, sr.g);
      m.b = colorDodge1(bd.b, sr.b);
      m.a = 0;
      RGBA8 f = alphaFix(bd, sr, m);
      return premultiply(f.r, f.g, f.b, f.a);
    }
    case OverlayBlend:  // :175-179
      r.r = hardLight(s.r, s.a, b.r, b.a);
      r.g = hardLight(s.g, s.a, b.g, b.a);
      r.b = hardLight(s.b, s.a, b.b, b.a);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case HardLightBlend:  // :184-188
      r.r = hardLight(b.r, b.a, s.r, s.a);
      r.g = hardLight(b.g, b.a, s.g, s.a);
      r.b = hardLight(b.b, b.a, s.b, s.a);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case DifferenceBlend:  // :190-204
      r.r = difference1(b.r, b.a, s.r, s.a);
      r.g = difference1(b.g, b.a, s.g, s.a);
      r.b = difference1(b.b, b.a, s.b, s.a);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case ExclusionBlend:  // :206-213
      r.r = exclusion1(b.r, s.r);
      r.g = exclusion1(b.g, s.g);
      r.b = exclusion1(b.b, s.b);
      r.a = blendAlpha(b.a, s.a);
      return r;
    case SoftLightBlend:
    case HueBlend:
    case SaturationBlend:
    case ColorBlend:
    case LuminosityBlend: return blendFloat(b, s, mode);
    case MaskBlend: {  // :227-232
      uint32_t k = s.a;
      return rgbx((b.r * k) / 255, (b.g * k) / 255, (b.b * k) / 255, (b.a * k) / 255);
    }
    case OverwriteBlend: return s;  // :266-267
    case SubtractMaskBlend: {       // :234-239
      uint32_t a = (b.a * (uint32_t)(uint8_t)(255 - s.a)) / 255;
      return rgbx((b.r * a) / 255, (b.g * a) / 255, (b.b * a) / 255, a);
    }
    case ExcludeMaskBlend: {  // :241-246
      uint32_t a = (uint32_t)std::max(b.a, s.a) - std::min(b.a, s.a);
      return rgbx((s.r * a) / 255, (s.g * a) / 255, (s.b * a) / 255, a);
    }
  }
  return b;
}

// ---------------------------------------------------------------------------
// Images  common.nim:34-57
// ---------------------------------------------------------------------------
struct Image {
  int64_t width, height;
  RGBX* data;  // borrowed, row-major, width*height
  int64_t idx(int64_t x, int64_t y) const { return width * y + x; }
  int64_t len() const { return width * height; }
};

// fillUnsafe  internal.nim:55-66.  Out-of-range or negative lengths, which
// corrupt memory or crash in the reference, are clamped to the buffer.
static void fillUnsafe(Image& img, RGBX c, int64_t start, int64_t len) {
  int64_t end = start + len;
  if (start < 0) start = 0;
  if (end > img.len()) end = img.len();
  for (int64_t i = start; i < end; i++) img.data[i] = c;
}
// clearUnsafe  paths.nim:1433-1440
static void clearUnsafe(Image& img, int64_t sx, int64_t sy, int64_t tx, int64_t ty) {
  if (sx == img.width || sy == img.height) return;
  int64_t start = img.idx(sx, sy);
  int64_t len = img.idx(tx, ty) - start;
  fillUnsafe(img, RGBX{0, 0, 0, 0}, start, len);
}

// ---------------------------------------------------------------------------
// Geometry (vmath / bumpy restated from the mathematical definitions)
// ---------------------------------------------------------------------------
struct Vec2 {
  float x, y;
};
static inline Vec2 v2(float x, float y) { return Vec2{x, y}; }
static inline Vec2 operator+(Vec2 a, Vec2 b) { return {a.x + b.x, a.y + b.y}; }
static inline Vec2 operator-(Vec2 a, Vec2 b) { return {a.x - b.x, a.y - b.y}; }
static inline Vec2 operator*(Vec2 a, float s) { return {a.x * s, a.y * s}; }
static inline Vec2 operator/(Vec2 a, float s) { return {a.x / s, a.y / s}; }
static inline bool operator==(Vec2 a, Vec2 b) { return a.x == b.x && a.y == b.y; }
static inline bool operator!=(Vec2 a, Vec2 b) { return !(a == b); }
static inline float lengthSq(Vec2 v) { return v.x * v.x + v.y * v.y; }  // vmath lengthSq
static inline float length(Vec2 v) { return sqrtf(lengthSq(v)); }       // vmath length
static inline Vec2 normalize(Vec2 v) { return v / length(v); }          // vmath normalize: v / |v|

struct Segment {
  Vec2 at, to;
};

// Mat3, column-major like vmath: m[col*3+row]; translation in m[6], m[7].
struct Mat3 {
  float m[9];
};
static inline Vec2 mul(const Mat3& M, Vec2 v) {  // vmath Mat3 * Vec2
  return v2(M.m[0] * v.x + M.m[3] * v.y + M.m[6], M.m[1] * v.x + M.m[4] * v.y + M.m[7]);
}
static inline bool is_identity(const Mat3& M) {
  static const float I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 9; i++)
    if (!(M.m[i] == I[i])) return false;
  return true;
}
static inline float pixelScale(const Mat3& M) {  // paths.nim:61-66
  return nmax(length(v2(M.m[0], M.m[1])), length(v2(M.m[3], M.m[4])));
}

// bumpy `intersects(Segment, Line, at)`: intersection of a segment with an
// infinite line, as used to clip band-spanning entries (paths.nim:1240-1247).
// bumpy is not vendored; restated with the parametric form that pixie's own
// copy for two segments uses (internal.nim:36-48), without the range check on
// the line's parameter; the point is taken on the segment (at + t*s1).
static bool intersectSegLine(Segment s, Vec2 l0, Vec2 l1, Vec2& at) {
  Vec2 s1 = s.to - s.at;
  Vec2 s2 = l1 - l0;
  float den = (-s2.x * s1.y + s1.x * s2.y);
  float t = (s2.x * (s.at.y - l0.y) - s2.y * (s.at.x - l0.x)) / den;
  if (t >= 0 && t <= 1) {
    at = s.at + s1 * t;
    return true;
  }
  return false;
}
// pixie's intersectsInside  internal.nim:36-48
static bool intersectsInside(Segment a, Segment b, Vec2& at) {
  Vec2 s1 = a.to - a.at;
  Vec2 s2 = b.to - b.at;
  float den = (-s2.x * s1.y + s1.x * s2.y);
  float s = (-s1.y * (a.at.x - b.at.x) + s1.x * (a.at.y - b.at.y)) / den;
  float t = (s2.x * (a.at.y - b.at.y) - s2.y * (a.at.x - b.at.x)) / den;
  if (s > 0 && s < 1 && t > 0 && t < 1) {
    at = a.at + s1 * t;
    return true;
  }
  return false;
}
// bumpy `intersects(Line, Line, at)` (miter joins, paths.nim:1993-1997):
// infinite lines, same parametric form.
static bool intersectLines(Vec2 a0, Vec2 a1, Vec2 b0, Vec2 b1, Vec2& at) {
  Vec2 s1 = a1 - a0;
  Vec2 s2 = b1 - b0;
  float den = (-s2.x * s1.y + s1.x * s2.y);
  if (den == 0) return false;
  float t = (s2.x * (a0.y - b0.y) - s2.y * (a0.x - b0.x)) / den;
  at = a0 + s1 * t;
  return true;
}
// vmath quantize(v, n) = sign(v) * floor(|v| / n) * n  (truncation toward 0).
static inline float quantize(float v, float n) {
  float sgn = v >= 0 ? 1.0f : -1.0f;
  return sgn * (floorf(fabsf(v) / n) * n);
}
// vmath fractional(v): fractional part of |v|.
static inline float fractional(float v) {
  float a = fabsf(v);
  return a - floorf(a);
}
// vmath angle(v) = atan2(y, x); fixAngle wraps into [-PI, PI].
static inline float angleOf(Vec2 v) { return atan2f(v.y, v.x); }
// Nim typing: a float32 compared with the float64 constant PI is promoted to
// float64; the compound assignment narrows the constant to float32.
static inline float fixAngle(float a) {
  const float tau = (float)(kPI * 2);
  while ((double)a > kPI) a -= tau;
  while ((double)a < -kPI) a += tau;
  return a;
}

// ---------------------------------------------------------------------------
// commandsToShapes  paths.nim:654-1057
// ---------------------------------------------------------------------------
enum Cmd {
  Close = 0, Move, Line, HLine, VLine, Cubic, SCubic, Quad, TQuad, Arc,
  RMove, RLine, RHLine, RVLine, RCubic, RSCubic, RQuad, RTQuad, RArc
};
static int paramCount(int k) {  // paths.nim:72-81
  switch (k) {
    case Close: return 0;
    case Move: case Line: case RMove: case RLine: case TQuad: case RTQuad: return 2;
    case HLine: case VLine: case RHLine: case RVLine: return 1;
    case Cubic: case RCubic: return 6;
    case SCubic: case RSCubic: case Quad: case RQuad: return 4;
    case Arc: case RArc: return 7;
  }
  return -1;
}

using Polygon = std::vector<Vec2>;

static void addSegment(Polygon& shape, Vec2 at, Vec2 to) {  // paths.nim:669-675
  if ((at - to) != v2(0, 0)) {
    if (shape.empty() || shape.back() != at) shape.push_back(at);
    shape.push_back(to);
  }
}

static inline Vec2 cubicAt(Vec2 a, Vec2 c1, Vec2 c2, Vec2 to, float t) {  // :679-686
  float t2 = t * t, t3 = t2 * t;
  return a * (((-t3 + 3 * t2) - 3 * t) + 1) + c1 * ((3 * t3 - 6 * t2) + 3 * t) +
         c2 * (-3 * t3 + 3 * t2) + to * (t3);
}
static inline Vec2 cubicDeriv(Vec2 a, Vec2 c1, Vec2 c2, Vec2 to, float t) {  // :688-693
  float t2 = t * t;
  return a * ((-3 * t2 + 6 * t) - 3) + c1 * ((9 * t2 - 12 * t) + 3) + c2 * (-9 * t2 + 6 * t) +
         to * (3 * t2);
}
static void addCubic(Polygon& shape, Vec2 at, Vec2 c1, Vec2 c2, Vec2 to, float ems) {  // :677-723
  float t = 0, step = 1;
  Vec2 prev = at;
  Vec2 next = cubicAt(at, c1, c2, to, t + step);
  Vec2 halfway = cubicAt(at, c1, c2, to, t + step / 2);
  while (true) {
    if (step <= FLT_EPSILON) throw PixieError("Unable to discretize cubic");
    Vec2 midpoint = (prev + next) / 2;
    Vec2 lineTangent = midpoint - prev;
    Vec2 curveTangent = cubicDeriv(at, c1, c2, to, t + step / 2);
    Vec2 curveTangentScaled = normalize(curveTangent) * length(lineTangent);
    float error = lengthSq(midpoint - halfway);
    float errorTangent = lengthSq(lineTangent - curveTangentScaled);
    if (error + errorTangent > ems) {
      next = halfway;
      halfway = cubicAt(at, c1, c2, to, t + step / 4);
      step /= 2;
    } else {
      addSegment(shape, prev, next);
      t += step;
      if (t == 1) break;
      prev = next;
      step = nmin(step * 2, 1 - t);
      next = cubicAt(at, c1, c2, to, t + step);
      halfway = cubicAt(at, c1, c2, to, t + step / 2);
    }
  }
}
static inline Vec2 quadAt(Vec2 a, Vec2 c, Vec2 to, float t) {  // :727-731
  float t2 = t * t;
  return a * ((t2 - 2 * t) + 1) + c * (-2 * t2 + 2 * t) + to * t2;
}
static void addQuadratic(Polygon& shape, Vec2 at, Vec2 c, Vec2 to, float ems) {  // :725-762
  float t = 0, step = 1;
  Vec2 prev = at;
  Vec2 next = quadAt(at, c, to, t + step);
  Vec2 halfway = quadAt(at, c, to, t + step / 2);
  bool halfStepping = false;
  while (true) {
    if (step <= FLT_EPSILON) throw PixieError("Unable to discretize quadratic");
    Vec2 midpoint = (prev + next) / 2;
    float error = lengthSq(midpoint - halfway);
    if (error > ems) {
      next = halfway;
      halfway = quadAt(at, c, to, t + step / 4);
      halfStepping = true;
      step /= 2;
    } else {
      addSegment(shape, prev, next);
      t += step;
      if (t == 1) break;
      prev = next;
      if (halfStepping)
        step = nmin(step, 1 - t);
      else
        step = nmin(step * 2, 1 - t);
      next = quadAt(at, c, to, t + step);
      halfway = quadAt(at, c, to, t + step / 2);
    }
  }
}

// Arc  paths.nim:764-884.  Nim typing: a float32 operand meeting the float64
// constant PI (or 2*PI) is promoted to float64 and narrowed back on
// assignment to a float32; compound assignments narrow the constant instead.
// cos/sin/arccos/sqrt of float32 are cosf/sinf/acosf/sqrtf.  This typing is
// pinned by the reference's polygon/arc goldens.
struct ArcParams {
  Vec2 radii;
  float rc, rs;  // rotation cos/sin (rotMat = rotate(radians))
  Vec2 center;
  float theta, delta;
};
static float svgAngle(Vec2 u, Vec2 v) {  // :809-815
  float d = u.x * v.x + u.y * v.y;
  float len = length(u) * length(v);
  float q = d / len;
  float c = q < -1 ? -1 : (q > 1 ? 1 : q);  // clamp
  float r = acosf(c);
  if ((u.x * v.y - u.y * v.x) < 0) r = -r;
  return r;
}
static ArcParams endpointToCenter(Vec2 at, Vec2 radiiIn, float rotation, bool large, bool sweep,
                                  Vec2 to) {  // :778-846
  Vec2 radii = v2(fabsf(radiiIn.x), fabsf(radiiIn.y));
  Vec2 radiiSq = v2(radii.x * radii.x, radii.y * radii.y);
  float radians = (float)((double)(rotation / 180.0f) * kPI);
  float cr_ = cosf(radians), sr_ = sinf(radians);
  Vec2 d = v2((at.x - to.x) / 2.0f, (at.y - to.y) / 2.0f);
  Vec2 p = v2(cr_ * d.x + sr_ * d.y, -sr_ * d.x + cr_ * d.y);
  Vec2 pSq = v2(p.x * p.x, p.y * p.y);
  float cr = pSq.x / radiiSq.x + pSq.y / radiiSq.y;
  if (cr > 1) {
    radii = radii * sqrtf(cr);
    radiiSq = v2(radii.x * radii.x, radii.y * radii.y);
  }
  float dq = radiiSq.x * pSq.y + radiiSq.y * pSq.x;
  float pq = (radiiSq.x * radiiSq.y - dq) / dq;
  float q = sqrtf(nmax(0, pq));
  if (large == sweep) q = -q;
  Vec2 cp = v2(q * radii.x * p.y / radii.y, -q * radii.y * p.x / radii.x);
  Vec2 center = v2(cr_ * cp.x - sr_ * cp.y + (at.x + to.x) / 2,
                   sr_ * cp.x + cr_ * cp.y + (at.y + to.y) / 2);
  float theta = svgAngle(v2(1, 0), v2((p.x - cp.x) / radii.x, (p.y - cp.y) / radii.y));
  float delta = svgAngle(v2((p.x - cp.x) / radii.x, (p.y - cp.y) / radii.y),
                         v2((-p.x - cp.x) / radii.x, (-p.y - cp.y) / radii.y));
  const float tau = (float)(kPI * 2);
  delta = (float)fmod((double)delta, kPI * 2);
  if (sweep && delta < 0)
    delta += tau;
  else if (!sweep && delta > 0)
    delta -= tau;
  while ((double)delta > kPI * 2) delta -= tau;
  while ((double)delta < -kPI * 2) delta += tau;
  ArcParams a;
  a.radii = radii;
  a.rc = cosf(radians);
  a.rs = sinf(radians);
  a.center = center;
  a.theta = theta;
  a.delta = delta;
  return a;
}
// rotMat * v + center (:848-850); rotate(radians) maps (x, y) to
// (c*x - s*y, s*x + c*y) (the other orientation fails the rotated-arc golden).
static inline Vec2 arcAt(const ArcParams& a, float ang) {
  Vec2 r = v2(cosf(ang) * a.radii.x, sinf(ang) * a.radii.y);
  Mat3 M;
  float m[9] = {a.rc, a.rs, 0, -a.rs, a.rc, 0, 0, 0, 1};
  memcpy(M.m, m, sizeof m);
  return mul(M, r) + a.center;
}
static void addArc(Polygon& shape, Vec2 at, Vec2 radii, float rotation, bool large, bool sweep,
                   Vec2 to, float ems) {  // :764-884
  ArcParams arc = endpointToCenter(at, radii, rotation, large, sweep, to);
  float t = 0, step = 1;
  Vec2 prev = at;
  while (t != 1) {
    if (step <= FLT_EPSILON) throw PixieError("Unable to discretize arc");
    float aPrev = arc.theta + arc.delta * t;
    float a = arc.theta + arc.delta * (t + step);
    Vec2 next = arcAt(arc, a);
    Vec2 halfway = arcAt(arc, aPrev + (a - aPrev) / 2);
    Vec2 midpoint = (prev + next) / 2;
    float error = lengthSq(midpoint - halfway);
    if (error > ems) {
      Vec2 quarterway = arcAt(arc, aPrev + (a - aPrev) / 4);
      Vec2 mid2 = (prev + halfway) / 2;
      float halfwayError = lengthSq(mid2 - quarterway);
      if (halfwayError < ems) {
        addSegment(shape, prev, halfway);
        prev = halfway;
        t += step / 2;
        step = nmin(step / 2, 1 - t);
      } else {
        step = step / 4;
      }
    } else {
      addSegment(shape, prev, next);
      prev = next;
      t += step;
      step = nmin(step * 2, 1 - t);
    }
  }
}

static std::vector<Polygon> commandsToShapes(const float* cmd, int64_t n, bool closeSubpaths,
                                             float pxScale) {  // :654-1057
  std::vector<Polygon> result;
  Vec2 start{0, 0}, at{0, 0};
  Polygon shape;
  int prevKind = Move;
  Vec2 prevCtrl{0, 0}, prevCtrl2{0, 0};
  float ems = powf(kPixelErrorMargin / pxScale, 2);
  int64_t i = 0;
  while (i < n) {
    int kind = (int)cmd[i];
    i++;
    const float* c = cmd + i;
    switch (kind) {
      case Move:
        if (!shape.empty()) {
          if (closeSubpaths) addSegment(shape, at, start);
          result.push_back(shape);
          shape.clear();
        }
        at = v2(c[0], c[1]);
        start = at;
        break;
      case Line: {
        Vec2 to = v2(c[0], c[1]);
        addSegment(shape, at, to);
        at = to;
      } break;
      case HLine: {
        Vec2 to = v2(c[0], at.y);
        addSegment(shape, at, to);
        at = to;
      } break;
      case VLine: {
        Vec2 to = v2(at.x, c[0]);
        addSegment(shape, at, to);
        at = to;
      } break;
      case Cubic: {
        Vec2 c1 = v2(c[0], c[1]), c2 = v2(c[2], c[3]), to = v2(c[4], c[5]);
        addCubic(shape, at, c1, c2, to, ems);
        at = to;
        prevCtrl2 = c2;
      } break;
      case SCubic: {
        Vec2 c2 = v2(c[0], c[1]), to = v2(c[2], c[3]);
        if (prevKind == Cubic || prevKind == SCubic || prevKind == RCubic || prevKind == RSCubic) {
          Vec2 c1 = at * 2 - prevCtrl2;
          addCubic(shape, at, c1, c2, to, ems);
        } else {
          addCubic(shape, at, at, c2, to, ems);
        }
        at = to;
        prevCtrl2 = c2;
      } break;
      case Quad: {
        Vec2 ctrl = v2(c[0], c[1]), to = v2(c[2], c[3]);
        addQuadratic(shape, at, ctrl, to, ems);
        at = to;
        prevCtrl = ctrl;
      } break;
      case TQuad: {
        Vec2 to = v2(c[0], c[1]);
        Vec2 ctrl = (prevKind == Quad || prevKind == TQuad || prevKind == RQuad || prevKind == RTQuad)
                        ? at * 2 - prevCtrl
                        : at;
        addQuadratic(shape, at, ctrl, to, ems);
        at = to;
        prevCtrl = ctrl;
      } break;
      case Arc: {
        Vec2 radii = v2(c[0], c[1]);
        float rot = c[2];
        bool large = c[3] == 1, sweep = c[4] == 1;
        Vec2 to = v2(c[5], c[6]);
        addArc(shape, at, radii, rot, large, sweep, to, ems);
        at = to;
      } break;
      case RMove:
        if (!shape.empty()) {
          result.push_back(shape);
          shape.clear();
        }
        at.x += c[0];
        at.y += c[1];
        start = at;
        break;
      case RLine: {
        Vec2 to = v2(at.x + c[0], at.y + c[1]);
        addSegment(shape, at, to);
        at = to;
      } break;
      case RHLine: {
        Vec2 to = v2(at.x + c[0], at.y);
        addSegment(shape, at, to);
        at = to;
      } break;
      case RVLine: {
        Vec2 to = v2(at.x, at.y + c[0]);
        addSegment(shape, at, to);
        at = to;
      } break;
      case RCubic: {
        Vec2 c1 = v2(at.x + c[0], at.y + c[1]), c2 = v2(at.x + c[2], at.y + c[3]),
             to = v2(at.x + c[4], at.y + c[5]);
        addCubic(shape, at, c1, c2, to, ems);
        at = to;
        prevCtrl2 = c2;
      } break;
      case RSCubic: {
        Vec2 c2 = v2(at.x + c[0], at.y + c[1]), to = v2(at.x + c[2], at.y + c[3]);
        Vec2 c1 = (prevKind == Cubic || prevKind == SCubic || prevKind == RCubic || prevKind == RSCubic)
                      ? at * 2 - prevCtrl2
                      : at;
        addCubic(shape, at, c1, c2, to, ems);
        at = to;
        prevCtrl2 = c2;
      } break;
      case RQuad: {
        Vec2 ctrl = v2(at.x + c[0], at.y + c[1]), to = v2(at.x + c[2], at.y + c[3]);
        addQuadratic(shape, at, ctrl, to, ems);
        at = to;
        prevCtrl = ctrl;
      } break;
      case RTQuad: {
        Vec2 to = v2(at.x + c[0], at.y + c[1]);
        Vec2 ctrl = (prevKind == Quad || prevKind == TQuad || prevKind == RQuad || prevKind == RTQuad)
                        ? at * 2 - prevCtrl
                        : at;
        addQuadratic(shape, at, ctrl, to, ems);
        at = to;
        prevCtrl = ctrl;
      } break;
      case RArc: {
        Vec2 radii = v2(c[0], c[1]);
        float rot = c[2];
        bool large = c[3] == 1, sweep = c[4] == 1;
        Vec2 to = v2(at.x + c[5], at.y + c[6]);
        addArc(shape, at, radii, rot, large, sweep, to, ems);
        at = to;
      } break;
      case Close:
        if (at != start) {
          addSegment(shape, at, start);
          at = start;
        }
        if (!shape.empty()) {
          result.push_back(shape);
          shape.clear();
        }
        break;
    }
    i += paramCount(kind);
    prevKind = kind;
  }
  if (!shape.empty()) {
    if (closeSubpaths) addSegment(shape, at, start);
    result.push_back(shape);
  }
  return result;
}

static void validateCommands(const float* cmd, int64_t n) {
  int64_t i = 0;
  while (i < n) {
    float f = cmd[i];
    if (!(f >= 0 && f <= 18) || f != floorf(f)) throw PixieError("Invalid path command");
    int pc = paramCount((int)f);
    if (i + 1 + pc > n) throw PixieError("Invalid path, wrong number of parameters");
    for (int k = 0; k < pc; k++)
      if (!std::isfinite(cmd[i + 1 + k])) throw PixieError("Invalid path, non-finite parameter");
    i += 1 + pc;
  }
}

static void transformShapes(std::vector<Polygon>& shapes, const Mat3& M) {  // :1092-1096
  if (is_identity(M)) return;
  for (auto& s : shapes)
    for (auto& v : s) v = mul(M, v);
}

// ---------------------------------------------------------------------------
// strokeShapes  paths.nim:1922-2082 (host side in the product too)
// ---------------------------------------------------------------------------
enum LineCap { ButtCap = 0, RoundCap, SquareCap };
enum LineJoin { MiterJoin = 0, RoundJoin, BevelJoin };

static const double kSplineCircleK = 4.0 * (-1.0 + 1.4142135623730951) / 3;  // :564 (float64)
static std::vector<float> ellipseCommands(float cx, float cy, float rx, float ry) {  // :604-616
  // magicX/magicY are float64 (float64 constant * float32); sums with them are
  // float64 and narrowed when passed to bezierCurveTo.
  double magicX = kSplineCircleK * (double)rx, magicY = kSplineCircleK * (double)ry;
  auto P = [](double v) { return (float)v; };
  return {(float)Move, cx + rx, cy,
          (float)Cubic, cx + rx, P(cy + magicY), P(cx + magicX), cy + ry, cx, cy + ry,
          (float)Cubic, P(cx - magicX), cy + ry, cx - rx, P(cy + magicY), cx - rx, cy,
          (float)Cubic, cx - rx, P(cy - magicY), P(cx - magicX), cy - ry, cx, cy - ry,
          (float)Cubic, P(cx + magicX), cy - ry, cx + rx, P(cy - magicY), cx + rx, cy,
          (float)Close};
}

static std::vector<Polygon> strokeShapes(const std::vector<Polygon>& shapes, float strokeWidth,
                                         int lineCap, int lineJoin, float miterLimit,
                                         std::vector<float> dashesIn, float pxScale) {
  std::vector<Polygon> result;
  if (strokeWidth <= 0) return result;
  const float halfStroke = strokeWidth / 2;
  const float miterAngleLimit = asinf(1 / miterLimit) * 2;  // miterLimitToAngle :1914-1916

  auto makeCircle = [&](Vec2 at) -> Polygon {  // :1938-1941
    auto cmds = ellipseCommands(at.x, at.y, halfStroke, halfStroke);
    return commandsToShapes(cmds.data(), (int64_t)cmds.size(), true, pxScale)[0];
  };
  auto makeRect = [&](Vec2 at, Vec2 to) -> Polygon {  // :1943-1965
    Vec2 tangent = normalize(to - at);
    Vec2 normal = v2(tangent.y, tangent.x);
    Vec2 a = v2(at.x + normal.x * halfStroke, at.y - normal.y * halfStroke);
    Vec2 b = v2(to.x + normal.x * halfStroke, to.y - normal.y * halfStroke);
    Vec2 c = v2(to.x - normal.x * halfStroke, to.y + normal.y * halfStroke);
    Vec2 d = v2(at.x - normal.x * halfStroke, at.y + normal.y * halfStroke);
    return Polygon{a, b, c, d, a};
  };
  auto addJoin = [&](std::vector<Polygon>& out, Vec2 prevPos, Vec2 pos, Vec2 nextPos) {  // :1967-2013
    float minArea = kPixelErrorMargin / pxScale;
    if (lineJoin == RoundJoin) {
      float area = (float)kPI * halfStroke * halfStroke;
      if (area > minArea) out.push_back(makeCircle(pos));
      return;
    }
    float angle = fixAngle(angleOf(nextPos - pos) - angleOf(prevPos - pos));
    if (fabs((double)fabsf(angle) - kPI) > (double)kEpsilon) {
      Vec2 a = normalize(pos - prevPos) * halfStroke;
      Vec2 b = normalize(pos - nextPos) * halfStroke;
      if (angle >= 0) {
        a = v2(-a.y, a.x);
        b = v2(b.y, -b.x);
      } else {
        a = v2(a.y, -a.x);
        b = v2(-b.y, b.x);
      }
      int lj = lineJoin;
      if (lj == MiterJoin && fabsf(angle) < miterAngleLimit) lj = BevelJoin;
      if (lj == MiterJoin) {
        Vec2 at;
        if (intersectLines(prevPos + a, pos + a, nextPos + b, pos + b, at)) {
          float bisectorLengthSq = lengthSq(at - pos);
          float areaSq = 0.25f * (lengthSq(a) * bisectorLengthSq + lengthSq(b) * bisectorLengthSq);
          if (areaSq > (minArea * minArea)) out.push_back(Polygon{pos + a, at, pos + b, pos, pos + a});
        }
      } else if (lj == BevelJoin) {
        float areaSq = 0.25f * lengthSq(a) * lengthSq(b);
        if (areaSq > (minArea * minArea)) out.push_back(Polygon{a + pos, b + pos, pos, a + pos});
      }
    }
  };

  for (const Polygon& shape : shapes) {  // :2015-2082
    std::vector<Polygon> shapeStroke;
    if (shape[0] != shape.back()) {
      if (lineCap == RoundCap) {
        shapeStroke.push_back(makeCircle(shape[0]));
      } else if (lineCap == SquareCap) {
        Vec2 tangent = normalize(shape[1] - shape[0]);
        shapeStroke.push_back(makeRect(shape[0] - tangent * halfStroke, shape[0]));
      }
    }
    std::vector<float> dashes = dashesIn;
    if (dashes.size() % 2 != 0) {
      std::vector<float> d2 = dashes;
      dashes.insert(dashes.end(), d2.begin(), d2.end());
    }
    for (float d : dashes)
      if (d <= 0.0f) throw PixieError("Invalid line dash value");
    for (size_t i = 1; i < shape.size(); i++) {
      Vec2 pos = shape[i], prevPos = shape[i - 1];
      if (!dashes.empty()) {
        float distance = length(prevPos - pos);   // dist(prevPos, pos)
        Vec2 dir = normalize(pos - prevPos);      // dir(pos, prevPos)
        Vec2 currPos = prevPos;
        bool done = false;
        while (!done) {
          for (size_t j = 0; j < dashes.size(); j++) {
            float d = dashes[j];
            if (j % 2 == 0) {
              float dd = nmin(distance, d);
              shapeStroke.push_back(makeRect(currPos, currPos + dir * dd));
            }
            currPos = currPos + dir * d;
            distance -= d;
            if (distance <= 0) {
              done = true;
              break;
            }
          }
        }
      } else {
        shapeStroke.push_back(makeRect(prevPos, pos));
      }
      if (i < shape.size() - 1) addJoin(shapeStroke, prevPos, pos, shape[i + 1]);
    }
    if (shape[0] == shape.back()) {
      addJoin(shapeStroke, shape[shape.size() - 2], shape.back(), shape[1]);
    } else {
      if (lineCap == RoundCap) {
        shapeStroke.push_back(makeCircle(shape.back()));
      } else if (lineCap == SquareCap) {
        Vec2 tangent = normalize(shape.back() - shape[shape.size() - 2]);
        shapeStroke.push_back(makeRect(shape.back() + tangent * halfStroke, shape.back()));
      }
    }
    result.insert(result.end(), shapeStroke.begin(), shapeStroke.end());
  }
  return result;
}

// ---------------------------------------------------------------------------
// Segments and partitions  paths.nim:1059-1262
// ---------------------------------------------------------------------------
struct WSeg {
  Segment s;
  int16_t w;
};
static std::vector<WSeg> shapesToSegments(const std::vector<Polygon>& shapes) {  // :1059-1090
  std::vector<WSeg> out;
  const float q = 1.0f / 256;
  for (const Polygon& poly : shapes) {
    Vec2 vec1 = v2(poly.back().x, quantize(poly.back().y, q));
    for (size_t i = 0; i < poly.size(); i++) {
      Vec2 vec2 = v2(poly[i].x, quantize(poly[i].y, q));
      if (i == 0 && vec1 == vec2) continue;
      Segment seg{vec1, vec2};
      vec1 = vec2;
      if (seg.at.y == seg.to.y) continue;
      int16_t w = 1;
      if (seg.at.y > seg.to.y) {
        std::swap(seg.at, seg.to);
        w = -1;
      }
      out.push_back(WSeg{seg, w});
    }
  }
  return out;
}

struct RectF {
  float x, y, w, h;
};
static RectF computeBounds(const std::vector<WSeg>& segs) {  // :1098-1117
  float xMin = INFINITY, xMax = -INFINITY, yMin = INFINITY, yMax = -INFINITY;
  for (const WSeg& s : segs) {
    xMin = nmin(xMin, nmin(s.s.at.x, s.s.to.x));
    xMax = nmax(xMax, nmax(s.s.at.x, s.s.to.x));
    yMin = nmin(yMin, s.s.at.y);
    yMax = nmax(yMax, s.s.to.y);
  }
  RectF r{0, 0, 0, 0};
  if (std::isnan(xMin) || std::isnan(xMax) || std::isnan(yMin) || std::isnan(yMax)) return r;
  r.x = xMin;
  r.y = yMin;
  r.w = xMax - xMin;
  r.h = yMax - yMin;
  return r;
}
static RectF snapToPixels(RectF r) {  // common.nim:92-101
  float xMin = r.x, xMax = r.x + r.w, yMin = r.y, yMax = r.y + r.h;
  RectF o;
  o.x = floorf(xMin);
  o.w = ceilf(xMax) - o.x;
  o.y = floorf(yMin);
  o.h = ceilf(yMax) - o.y;
  return o;
}

struct Entry {  // PartitionEntry paths.nim:28-31
  Segment segment;
  float m, b;
  int16_t winding;
};
struct Partition {  // paths.nim:33-36
  std::vector<Entry> entries;
  bool requiresAntiAliasing = false, twoNonintersectingSpanningSegments = false;
  int64_t top = 0, bottom = 0;
};
static Entry initEntry(Segment s, int16_t w) {  // :1127-1135
  Entry e;
  e.segment = s;
  e.winding = w;
  e.m = 0;
  e.b = 0;
  float d = s.at.x - s.to.x;
  if (d == 0) {
    e.b = s.at.x;
  } else {
    e.m = (s.at.y - s.to.y) / d;
    e.b = s.at.y - e.m * s.at.x;
  }
  return e;
}
static inline float solveX(const Entry& e, float y) { return e.m == 0 ? e.b : (y - e.b) / e.m; }
static inline float solveY(const Entry& e, float x) { return e.m * x + e.b; }
static inline float midpointX(Segment s) { return (s.at.x + s.to.x) * 0.5f; }
static inline bool hasFractional(float v) { return v - truncf(v) != 0; }
static inline bool segRequiresAA(Segment s) {  // :1149-1160
  return s.at.x != s.to.x || hasFractional(s.at.x) || hasFractional(s.at.y) ||
         hasFractional(s.to.y);
}

static std::vector<Partition> partitionSegments(const std::vector<WSeg>& segs, int64_t top,
                                                int64_t height) {  // :1168-1262
  uint32_t maxP = (uint32_t)std::max<int64_t>(1, height / 4);
  uint32_t numP = std::min<uint32_t>(maxP, (uint32_t)std::max<int64_t>(1, (int64_t)segs.size() / 2));
  std::vector<Partition> res(numP);
  uint32_t startY = (uint32_t)top;
  uint32_t ph = (uint32_t)height / numP;
  res[0].top = top;
  res[0].bottom = top + (int64_t)ph;
  for (size_t i = 1; i < res.size(); i++) {
    res[i].top = res[i - 1].bottom;
    res[i].bottom = res[i - 1].bottom + (int64_t)ph;
  }
  res.back().bottom = top + height;

  if (numP == 1) {
    for (const WSeg& s : segs) res[0].entries.push_back(initEntry(s.s, s.w));
  } else {
    for (const WSeg& s : segs) {
      uint32_t a = nim_u32(nmax(0, s.s.at.y - (float)startY));
      uint32_t b = nim_u32(nmax(0, s.s.to.y - (float)startY));
      a = std::min(a / ph, numP - 1);
      b = std::min(b / ph, numP - 1);
      Entry e = initEntry(s.s, s.w);
      for (uint32_t k = a; k <= b; k++) res[k].entries.push_back(e);
    }
  }
  for (Partition& p : res) {
    p.requiresAntiAliasing = false;
    for (const Entry& e : p.entries)
      if (segRequiresAA(e.segment)) {
        p.requiresAntiAliasing = true;
        break;
      }
    float ptop = (float)p.top, pbot = (float)p.bottom;
    for (Entry& e : p.entries) {
      if (e.segment.at.y <= ptop && e.segment.to.y >= pbot) {
        Vec2 at{0, 0};
        intersectSegLine(e.segment, v2(0, ptop), v2(1000, ptop), at);
        e.segment.at = at;
        intersectSegLine(e.segment, v2(0, pbot), v2(1000, pbot), at);
        e.segment.to = at;
      }
    }
    if (p.entries.size() == 2) {
      Segment e0 = p.entries[0].segment, e1 = p.entries[1].segment;
      Vec2 at;
      if (!intersectsInside(e0, e1, at)) {
        if (e0.at.y <= ptop && e0.to.y >= pbot && e1.at.y <= ptop && e1.to.y >= pbot) {
          p.twoNonintersectingSpanningSegments = true;
          if (midpointX(e0) > midpointX(e1)) std::swap(p.entries[0], p.entries[1]);
        }
      }
    }
  }
  return res;
}

// ---------------------------------------------------------------------------
// Scan conversion  paths.nim:1264-1912
// ---------------------------------------------------------------------------
typedef int32_t Fixed32;
static inline Fixed32 fixed32(float f) { return nim_i32(f * 256); }  // :1267-1268
static inline int64_t integerOf(Fixed32 p) { return p / 256; }        // :1270-1271
static inline Fixed32 truncFx(Fixed32 p) { return (p / 256) * 256; }  // :1273-1274

struct Hit {
  Fixed32 x;
  int16_t w;
};
static void sortHits(std::vector<Hit>& hits, int len) {  // :1277-1286
  for (int i = 1; i < len; i++) {
    int j = i - 1, k = i;
    while (j >= 0 && hits[j].x > hits[k].x) {
      std::swap(hits[j + 1], hits[j]);
      j--;
      k--;
    }
  }
}
static inline bool shouldFill(int rule, int64_t count) {  // :1288-1296
  return rule == 0 ? count != 0 : (count % 2 != 0);
}
struct Span {
  Fixed32 prevAt, at;
  int64_t count;
};
static void walk(const std::vector<Hit>& hits, int numHits, int rule,
                 std::vector<Span>& out) {  // :1298-1334
  out.clear();
  int i = 0;
  int64_t count = 0;
  Fixed32 prevAt = 0;
  while (i < numHits) {
    Fixed32 at = hits[i].x;
    int16_t winding = hits[i].w;
    if (at > 0) {
      if (shouldFill(rule, count)) {
        if (i < numHits - 1) {
          Fixed32 nextAt = hits[i + 1].x;
          int16_t nextW = hits[i + 1].w;
          if (nextAt == at && winding + nextW == 0) {
            i += 2;
            continue;
          }
          if (rule == 0 && count + winding != 0) {
            count += winding;
            i++;
            continue;
          }
        }
        out.push_back(Span{prevAt, at, count});
      }
      prevAt = at;
    }
    count += winding;
    i++;
  }
}

// The coverage row: writes outside [0, pathWidth) are undefined behaviour in
// the reference (checks are off); they are dropped here.
struct CovRow {
  std::vector<uint8_t> c;
  int64_t startX;
  void add(int64_t x, uint8_t v) {
    int64_t i = x - startX;
    if (i >= 0 && i < (int64_t)c.size()) c[(size_t)i] = (uint8_t)(c[(size_t)i] + v);
  }
};

static void computeCoverage(CovRow& cov, std::vector<Hit>& hits, int& numHits, int64_t width,
                            int64_t y, const Partition& part, const std::vector<int>& entryIdx,
                            int numEntryIdx, int rule, std::vector<Span>& spans) {  // :1350-1431
  bool aa = part.requiresAntiAliasing;
  int quality = aa ? 5 : 1;
  uint8_t sampleCoverage = (uint8_t)(255 / quality);
  float offset = 1 / (float)quality;
  float initialOffset = offset / 2 + kEpsilon;
  float yLine = (float)y + initialOffset - offset;
  for (int m = 0; m < quality; m++) {
    yLine += offset;
    numHits = 0;
    for (int i = 0; i < numEntryIdx; i++) {
      const Entry& e = part.entries[(size_t)entryIdx[(size_t)i]];
      if (e.segment.at.y <= yLine && e.segment.to.y >= yLine) {
        float x = e.m == 0 ? e.b : (yLine - e.b) / e.m;
        hits[(size_t)numHits] = Hit{fixed32(nmin(x, (float)width)), e.winding};
        numHits++;
      }
    }
    if (numHits > 0) sortHits(hits, numHits);
    if (aa) {
      walk(hits, numHits, rule, spans);
      for (const Span& sp : spans) {
        Fixed32 prevAt = sp.prevAt, at = sp.at;
        int64_t fillStart = integerOf(prevAt);
        bool pixelCrossed = integerOf(at) != integerOf(prevAt);
        Fixed32 leftCover = pixelCrossed ? truncFx(prevAt) + 256 - prevAt : at - prevAt;
        if (leftCover != 0) {
          fillStart++;
          cov.add(integerOf(prevAt), (uint8_t)integerOf(leftCover * (int32_t)sampleCoverage));
        }
        if (pixelCrossed) {
          Fixed32 rightCover = at - truncFx(at);
          if (rightCover > 0)
            cov.add(integerOf(at), (uint8_t)integerOf(rightCover * (int32_t)sampleCoverage));
        }
        int64_t fillLen = integerOf(at) - fillStart;
        if (fillLen > 0)
          for (int64_t j = fillStart; j < fillStart + fillLen; j++) cov.add(j, sampleCoverage);
      }
    }
  }
}

// applyOpacity(M128, float32) of the x86 SSE2 build (golden-pinning mode).
static inline RGBX opacity_sse2(RGBX c, float area) {  // applyOpacity(M128, float32) sse2.nim:6-11
  auto ch = [&](uint8_t v) -> uint32_t {
    float f = nearbyintf((float)v * area);
    if (!(f > 0)) return 0;
    return f > 255 ? 255u : (uint32_t)f;
  };
  return rgbx(ch(c.r), ch(c.g), ch(c.b), ch(c.a));
}

// ---------------------------------------------------------------------------
// The NEON line kernels (simd/neon.nim:427-700), TIMED CPU BASELINE ONLY (see
// simd_lines.h): with g_simd_variant = 1 the Normal/Mask/Overwrite lines of
// fills and of draw run these instead of the scalar loops.  Never set by the
// parity tests; bench.py times both variants.
// ---------------------------------------------------------------------------
int g_simd_variant = 0;

namespace nl {
using simd::u8x16;
static inline bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }
static inline u8x16 splat_px(RGBX c) {
  u8x16 v;
  for (int k = 0; k < 16; k += 4) {
    v[k] = c.r;
    v[k + 1] = c.g;
    v[k + 2] = c.b;
    v[k + 3] = c.a;
  }
  return v;
}
static inline u8x16 cov_bcast(u8x16 cv, int q) {  // coverage of pixels 4q..4q+3, each over its 4 bytes
  u8x16 v;
  for (int k = 0; k < 16; k++) v[k] = cv[4 * q + (k >> 2)];
  return v;
}
static inline bool all_bytes(u8x16 v, uint8_t x) {
  for (int k = 0; k < 16; k++)
    if (v[k] != x) return false;
  return true;
}
// blendLineNormalNeon(a, b)  :502-527
static void normal2(RGBX* a, const RGBX* b, int64_t len) {
  int64_t i = 0;
  for (; i < len && !aligned16(a + i); i++) a[i] = blendNormal(a[i], b[i]);
  for (; i < len - 16; i += 16) {
    u8x16 sv[4];
    bool opaque = true;
    for (int q = 0; q < 4; q++) {
      sv[q] = simd::load16(b + i + 4 * q);
      opaque = opaque && simd::all_alpha(sv[q], 255);
    }
    for (int q = 0; q < 4; q++)
      simd::store16(a + i + 4 * q, opaque ? sv[q] : simd::normal4(simd::load16(a + i + 4 * q), sv[q]));
  }
  for (; i < len; i++) a[i] = blendNormal(a[i], b[i]);
}
// blendLineMaskNeon(a, b)  :609-639
static void mask2(RGBX* a, const RGBX* b, int64_t len) {
  int64_t i = 0;
  for (; i < len && !aligned16(a + i); i++) a[i] = blend_px(MaskBlend, a[i], b[i]);
  for (; i < len - 16; i += 16) {
    u8x16 sv[4];
    bool opaque = true;
    for (int q = 0; q < 4; q++) {
      sv[q] = simd::load16(b + i + 4 * q);
      opaque = opaque && simd::all_alpha(sv[q], 255);
    }
    if (opaque) continue;
    for (int q = 0; q < 4; q++)
      simd::store16(a + i + 4 * q, simd::mul_div255(simd::load16(a + i + 4 * q), simd::alpha_bcast(sv[q])));
  }
  for (; i < len; i++) a[i] = blend_px(MaskBlend, a[i], b[i]);
}
// blendLineNormalNeon(line, rgbx)  :479-500
static void normal1(RGBX* a, RGBX c, int64_t len) {
  int64_t i = 0;
  for (; i < len && !aligned16(a + i); i++) a[i] = blendNormal(a[i], c);
  const u8x16 cv = splat_px(c);
  for (; i < len - 16; i += 16)
    for (int q = 0; q < 4; q++) simd::store16(a + i + 4 * q, simd::normal4(simd::load16(a + i + 4 * q), cv));
  for (; i < len; i++) a[i] = blendNormal(a[i], c);
}
// blendLineMaskNeon(line, rgbx)  :587-607
static void mask1(RGBX* a, RGBX c, int64_t len) {
  int64_t i = 0;
  for (; i < len && !aligned16(a + i); i++) a[i] = blend_px(MaskBlend, a[i], c);
  const u8x16 al = u8x16{} + c.a;
  for (; i < len - 16; i += 16)
    for (int q = 0; q < 4; q++) simd::store16(a + i + 4 * q, simd::mul_div255(simd::load16(a + i + 4 * q), al));
  for (; i < len; i++) a[i] = blend_px(MaskBlend, a[i], c);
}
// blendLineCoverage{Overwrite,Normal,Mask}Neon  :427-477, :529-585, :641-700
static void coverage(RGBX* line, const uint8_t* cov, RGBX c, int64_t len, int mode) {
  auto scalar = [&](int64_t i) {
    const uint8_t k = cov[i];
    if (mode == OverwriteBlend) {
      if (k != 0) line[i] = mul_c(c, k);
    } else if (mode == NormalBlend) {
      if (k != 0) line[i] = blendNormal(line[i], mul_c(c, k));
    } else {
      if (k == 0) line[i] = RGBX{0, 0, 0, 0};
      else if (k != 255) line[i] = blend_px(MaskBlend, line[i], mul_c(c, k));
    }
  };
  int64_t i = 0;
  for (; i < len && !aligned16(line + i); i++) scalar(i);
  const u8x16 cv = splat_px(c), al = u8x16{} + c.a;
  for (; i < len - 16; i += 16) {
    const u8x16 k = simd::load16(cov + i);
    const bool zero = all_bytes(k, 0), full = all_bytes(k, 255);
    if (mode == OverwriteBlend) {
      if (zero) continue;
      for (int q = 0; q < 4; q++)
        simd::store16(line + i + 4 * q, full ? cv : simd::mul_div255(cv, cov_bcast(k, q)));
    } else if (mode == NormalBlend) {
      if (zero) continue;
      for (int q = 0; q < 4; q++) {
        if (full && c.a == 255) {
          simd::store16(line + i + 4 * q, cv);
        } else {
          const u8x16 src = simd::mul_div255(cv, cov_bcast(k, q));
          simd::store16(line + i + 4 * q, simd::normal4(simd::load16(line + i + 4 * q), src));
        }
      }
    } else {
      if (zero) {
        for (int q = 0; q < 4; q++) simd::store16(line + i + 4 * q, u8x16{});
        continue;
      }
      if (full && c.a == 255) continue;
      for (int q = 0; q < 4; q++) {
        const u8x16 a = simd::mul_div255(al, cov_bcast(k, q));
        simd::store16(line + i + 4 * q, simd::mul_div255(simd::load16(line + i + 4 * q), a));
      }
    }
  }
  for (; i < len; i++) scalar(i);
}
}  // namespace nl

static void fillCoverage(Image& img, RGBX c, int64_t startX, int64_t y, const CovRow& cov,
                         int mode) {  // :1479-1526
  int64_t n = (int64_t)cov.c.size();
  RGBX* line = img.data + img.idx(startX, y);
  if (g_simd_variant && (mode == OverwriteBlend || mode == NormalBlend || mode == MaskBlend)) {
    nl::coverage(line, cov.c.data(), c, n, mode);
    if (mode == MaskBlend) {
      clearUnsafe(img, 0, y, startX, y);
      clearUnsafe(img, startX + n, y, img.width, y);
    }
    return;
  }
  switch (mode) {
    case OverwriteBlend:  // :1442-1451
      for (int64_t i = 0; i < n; i++)
        if (cov.c[(size_t)i] != 0) line[i] = mul_c(c, cov.c[(size_t)i]);
      break;
    case NormalBlend:  // :1453-1464
      for (int64_t i = 0; i < n; i++)
        if (cov.c[(size_t)i] != 0) line[i] = blendNormal(line[i], mul_c(c, cov.c[(size_t)i]));
      break;
    case MaskBlend:  // :1466-1477
      for (int64_t i = 0; i < n; i++)
        if (cov.c[(size_t)i] != 255) line[i] = blend_px(MaskBlend, line[i], mul_c(c, cov.c[(size_t)i]));
      clearUnsafe(img, 0, y, startX, y);
      clearUnsafe(img, startX + n, y, img.width, y);
      break;
    default:
      for (int64_t i = 0; i < n; i++)
        if (cov.c[(size_t)i] != 0) line[i] = blend_px(mode, line[i], mul_c(c, cov.c[(size_t)i]));
      break;
  }
}

static void fillHits(Image& img, RGBX c, int64_t startX, int64_t y, const std::vector<Hit>& hits,
                     int numHits, int rule, int mode, bool maskClears,
                     std::vector<Span>& spans) {  // :1540-1591
  walk(hits, numHits, rule, spans);
  auto forSpans = [&](auto fn) {  // walkInteger :1336-1348
    for (const Span& sp : spans) {
      int64_t fillStart = integerOf(sp.prevAt);
      int64_t fillLen = integerOf(sp.at) - fillStart;
      if (fillLen <= 0) continue;
      fn(fillStart, fillLen);
    }
  };
  switch (mode) {
    case OverwriteBlend:
      forSpans([&](int64_t s, int64_t l) { fillUnsafe(img, c, img.idx(s, y), l); });
      break;
    case NormalBlend:
      forSpans([&](int64_t s, int64_t l) {
        if (c.a == 255) {
          fillUnsafe(img, c, img.idx(s, y), l);
        } else if (g_simd_variant) {
          nl::normal1(img.data + img.idx(s, y), c, l);
        } else {
          RGBX* line = img.data + img.idx(s, y);
          for (int64_t i = 0; i < l; i++) line[i] = blendNormal(line[i], c);
        }
      });
      break;
    case MaskBlend: {
      int64_t filledTo = startX;
      forSpans([&](int64_t s, int64_t l) {
        if (maskClears) {
          int64_t gap = s - filledTo;
          if (gap > 0) fillUnsafe(img, RGBX{0, 0, 0, 0}, img.idx(filledTo, y), gap);
        }
        if (c.a != 255) {
          RGBX* line = img.data + img.idx(s, y);
          if (g_simd_variant) nl::mask1(line, c, l);
          else for (int64_t i = 0; i < l; i++) line[i] = blend_px(MaskBlend, line[i], c);
        }
        filledTo = s + l;
      });
      if (maskClears) {
        clearUnsafe(img, 0, y, startX, y);
        clearUnsafe(img, filledTo, y, img.width, y);
      }
    } break;
    default:
      forSpans([&](int64_t s, int64_t l) {
        RGBX* line = img.data + img.idx(s, y);
        for (int64_t i = 0; i < l; i++) line[i] = blend_px(mode, line[i], c);
      });
      break;
  }
}

// Row window of this thread (test infrastructure, not in the reference):
// fillShapes computes every row's geometry as usual but writes only rows in
// [g_row_lo, g_row_hi).  Rows are independent in the reference's row loop, so
// threads that each own a window and draw every path of a scene in order
// produce, together, the bytes of one thread drawing the whole canvas.
static thread_local int64_t g_row_lo = INT64_MIN, g_row_hi = INT64_MAX;

static void fillShapes(Image& img, const std::vector<Polygon>& shapes, RGBX c, int rule,
                       int mode) {  // :1593-1912
  std::vector<WSeg> segs = shapesToSegments(shapes);
  RectF bounds = snapToPixels(computeBounds(segs));
  int64_t startX = std::max<int64_t>(0, nim_int(bounds.x));
  int64_t startY = std::max<int64_t>(0, nim_int(bounds.y));
  int64_t pathWidth = startX < img.width ? std::min<int64_t>(nim_int(bounds.w), img.width - startX) : 0;
  int64_t pathHeight = std::min<int64_t>(img.height, nim_int(bounds.y + bounds.h));
  if (pathWidth == 0) return;
  if (pathWidth < 0) throw PixieError("Path int overflow detected");

  std::vector<Partition> parts = partitionSegments(segs, startY, pathHeight - startY);
  size_t maxEntries = 0;
  for (auto& p : parts) maxEntries = std::max(maxEntries, p.entries.size());
  std::vector<int> entryIdx(maxEntries);
  std::vector<Segment> trap(maxEntries);
  CovRow cov;
  cov.c.assign((size_t)pathWidth, 0);
  cov.startX = startX;
  std::vector<Hit> hits(maxEntries);
  std::vector<Span> spans;
  int numHits = 0;
  size_t pi = 0;
  const float W = (float)img.width;

  int64_t y = startY;
  while (y < pathHeight) {
    if (y >= parts[pi].bottom) pi++;
    Partition& part = parts[pi];
    int64_t pHeight = part.bottom - part.top;
    if (pHeight == 0) continue;

    if (part.twoNonintersectingSpanningSegments && !part.requiresAntiAliasing) {  // :1644-1668
      int64_t left = nim_int(part.entries[0].segment.at.x);
      int64_t right = nim_int(part.entries[1].segment.at.x);
      int64_t minX = std::min<int64_t>(std::max<int64_t>(left, 0), img.width);
      int64_t maxX = std::min<int64_t>(std::max<int64_t>(right, 0), img.width);
      bool skipBlending = mode == OverwriteBlend || (mode == NormalBlend && c.a == 255);
      if (skipBlending && minX == 0 && maxX == img.width) {
        const int64_t r0 = std::max(y, g_row_lo), r1 = std::min(y + pHeight, g_row_hi);
        if (r1 > r0) {
          int64_t start = img.idx(0, r0);
          int64_t len = img.idx(0, r1) - start;
          fillUnsafe(img, c, start, len);
        }
      } else {
        for (int64_t r = 0; r < pHeight; r++) {
          if (y + r < g_row_lo || y + r >= g_row_hi) continue;
          hits[0] = Hit{(Fixed32)(uint32_t)(minX * 256), 1};
          hits[1] = Hit{(Fixed32)(uint32_t)(maxX * 256), -1};
          fillHits(img, c, 0, y + r, hits, 2, 0, mode, true, spans);
        }
      }
      y += pHeight;
      continue;
    }

    if (y < g_row_lo || y >= g_row_hi) {  // another thread's row
      y++;
      continue;
    }
    float scanTop = (float)y, scanBottom = (float)(y + 1);
    bool allSpan = true;
    int numEntryIdx = 0;
    if (part.twoNonintersectingSpanningSegments) {
      numEntryIdx = 2;
      entryIdx[0] = 0;
      entryIdx[1] = 1;
    } else {
      for (size_t i = 0; i < part.entries.size(); i++) {
        const Segment& s = part.entries[i].segment;
        if (s.to.y <= scanTop || s.at.y >= scanBottom) continue;
        if (s.at.y > scanTop || s.to.y < scanBottom) allSpan = false;
        entryIdx[(size_t)numEntryIdx++] = (int)i;
      }
    }

    if (allSpan && numEntryIdx % 2 == 0) {  // trapezoids :1674-1872
      for (int i = 0; i < numEntryIdx; i++) {
        int k = entryIdx[(size_t)i];
        trap[(size_t)k].at.y = scanTop;
        trap[(size_t)k].to.y = scanBottom;
        trap[(size_t)k].at.x = solveX(part.entries[(size_t)k], scanTop);
        trap[(size_t)k].to.x = solveX(part.entries[(size_t)k], scanBottom);
      }
      bool noOverlap = true;
      for (int i = 1; i < numEntryIdx; i++) {
        int j = i - 1, k = i;
        while (j >= 0 && midpointX(trap[(size_t)entryIdx[(size_t)j]]) >
                             midpointX(trap[(size_t)entryIdx[(size_t)k]])) {
          std::swap(entryIdx[(size_t)j + 1], entryIdx[(size_t)j]);
          j--;
          k--;
        }
      }
      for (int i = 0; i < numEntryIdx - 1; i++) {
        Segment L = trap[(size_t)entryIdx[(size_t)i]], R = trap[(size_t)entryIdx[(size_t)i + 1]];
        float leftMaxX = nmax(L.at.x, L.to.x);
        float rightMinX = nmin(R.at.x, R.to.x);
        if (nim_int(ceilf(leftMaxX)) > nim_int(rightMinX)) {
          noOverlap = false;
          break;
        }
      }
      if (noOverlap) {
        bool simple = true;
        int64_t wc = 0;
        for (int i = 0; i < numEntryIdx; i += 2) {
          wc += part.entries[(size_t)entryIdx[(size_t)i]].winding;
          if (!shouldFill(rule, wc)) {
            simple = false;
            break;
          }
          wc += part.entries[(size_t)entryIdx[(size_t)i + 1]].winding;
          if (shouldFill(rule, wc)) {
            simple = false;
            break;
          }
        }
        if (simple) {
          int64_t filledTo = 0;
          for (int i = 0; i < numEntryIdx; i += 2) {
            const Entry& left = part.entries[(size_t)entryIdx[(size_t)i]];
            const Entry& right = part.entries[(size_t)entryIdx[(size_t)i + 1]];
            Segment trapLeft = trap[(size_t)entryIdx[(size_t)i]];
            Segment trapRight = trap[(size_t)entryIdx[(size_t)i + 1]];
            float leftMaxX = nmax(trapLeft.at.x, trapLeft.to.x);
            float rightMinX = nmin(trapRight.at.x, trapRight.to.x);
            int64_t leftCoverEnd = nim_int(ceilf(leftMaxX));
            int64_t rightCoverBegin = nim_int(truncf(rightMinX));
            {  // left sliver :1750-1788
              bool inverted = trapLeft.at.x < trapLeft.to.x;
              float sliverStart = nmin(trapLeft.at.x, trapLeft.to.x);
              float rectStart = leftMaxX;
              float pen = sliverStart, prevPen = pen;
              float penY = inverted ? (float)y : (float)(y + 1), prevPenY = penY;
              int64_t xEnd = nim_int(ceilf(rectStart));
              for (int64_t x = nim_int(sliverStart); x < xEnd; x++) {
                prevPen = pen;
                pen = (float)(x + 1);
                float rightRectArea = 0;
                if (pen > rectStart) {
                  rightRectArea = pen - rectStart;
                  pen = rectStart;
                }
                prevPenY = penY;
                penY = solveY(left, pen);
                if (x < 0 || x >= img.width) continue;
                float run = pen - prevPen;
                float triangleArea = 0.5f * run * fabsf(penY - prevPenY);
                float rectArea = inverted ? (prevPenY - (float)y) * run : ((float)(y + 1) - prevPenY) * run;
                float area = triangleArea + rectArea + rightRectArea;
                RGBX& px = img.data[img.idx(x, y)];
                px = blend_px(mode, px, g_golden_mode ? opacity_sse2(c, area) : mul_f(c, area));
              }
            }
            {  // right sliver :1790-1828
              bool inverted = trapRight.at.x > trapRight.to.x;
              float rectEnd = rightMinX;
              float sliverEnd = nmax(trapRight.at.x, trapRight.to.x);
              float pen = rectEnd, prevPen = pen;
              float penY = inverted ? (float)(y + 1) : (float)y, prevPenY = penY;
              int64_t xEnd = nim_int(ceilf(sliverEnd));
              for (int64_t x = nim_int(rectEnd); x < xEnd; x++) {
                prevPen = pen;
                pen = (float)(x + 1);
                float leftRectArea = fractional(prevPen);
                if (pen > sliverEnd) pen = sliverEnd;
                prevPenY = penY;
                penY = solveY(right, pen);
                if (x < 0 || x >= img.width) continue;
                float run = pen - prevPen;
                float triangleArea = 0.5f * run * fabsf(penY - prevPenY);
                float rectArea = inverted ? (penY - (float)y) * run : ((float)(y + 1) - penY) * run;
                float area = leftRectArea + triangleArea + rectArea;
                RGBX& px = img.data[img.idx(x, y)];
                px = blend_px(mode, px, g_golden_mode ? opacity_sse2(c, area) : mul_f(c, area));
              }
            }
            int64_t fillBegin = std::min<int64_t>(std::max<int64_t>(leftCoverEnd, 0), img.width);
            int64_t fillEnd = std::min<int64_t>(std::max<int64_t>(rightCoverBegin, 0), img.width);
            hits[0] = Hit{fixed32((float)fillBegin), 1};
            hits[1] = Hit{fixed32((float)fillEnd), -1};
            fillHits(img, c, 0, y, hits, 2, 0, mode, false, spans);
            if (mode == MaskBlend) {
              int64_t clearTo = nim_int(nmin(trapLeft.at.x, trapLeft.to.x));
              clearUnsafe(img, std::min<int64_t>(filledTo, img.width), y,
                          std::min<int64_t>(clearTo, img.width), y);
            }
            filledTo = nim_int(ceilf(nmax(trapRight.at.x, trapRight.to.x)));
          }
          if (mode == MaskBlend) clearUnsafe(img, std::min<int64_t>(filledTo, img.width), y, img.width, y);
          y++;
          continue;
        }
      }
    }

    computeCoverage(cov, hits, numHits, img.width, y, part, entryIdx, numEntryIdx, rule, spans);
    if (part.requiresAntiAliasing) {
      fillCoverage(img, c, startX, y, cov, mode);
      std::fill(cov.c.begin(), cov.c.end(), (uint8_t)0);
    } else {
      fillHits(img, c, startX, y, hits, numHits, rule, mode, true, spans);
    }
    y++;
  }
  (void)W;
  if (mode == MaskBlend) {
    const int64_t lo = std::max<int64_t>(g_row_lo, 0), hi = std::min<int64_t>(g_row_hi, img.height);
    if (lo == 0 && hi == img.height) {
      clearUnsafe(img, 0, 0, 0, startY);
      // rows [pathHeight, height); a negative pathHeight (path above the image)
      // is clamped to 0 where the reference writes before its buffer.
      clearUnsafe(img, 0, std::max<int64_t>(pathHeight, 0), 0, img.height);
    } else {  // the same rows, within the window
      if (std::min(startY, hi) > lo) clearUnsafe(img, 0, lo, 0, std::min(startY, hi));
      const int64_t b0 = std::max<int64_t>(std::max<int64_t>(pathHeight, 0), lo);
      if (hi > b0) clearUnsafe(img, 0, b0, 0, hi);
    }
  }
}

// ---------------------------------------------------------------------------
// fillPath / strokePath  paths.nim:2093-2175 (solid paint)
// ---------------------------------------------------------------------------
static void fillPath(Image& img, const float* cmds, int64_t n, const float color[4],
                     float opacity, int mode, const Mat3& M, int rule) {
  validateCommands(cmds, n);
  opacity = opacity < 0 ? 0 : (opacity > 1 ? 1 : opacity);  // clamp :2101
  if (opacity == 0) return;
  if (!(color[3] > 0 || mode == OverwriteBlend)) return;
  std::vector<Polygon> shapes = commandsToShapes(cmds, n, true, pixelScale(M));
  transformShapes(shapes, M);
  float c[4] = {color[0], color[1], color[2], color[3] * opacity};
  fillShapes(img, shapes, color_to_rgbx(c), rule, mode);
}
static void strokePath(Image& img, const float* cmds, int64_t n, const float color[4],
                       float opacity, int mode, const Mat3& M, float strokeWidth, int cap,
                       int join, float miterLimit, const float* dashes, int nd) {
  validateCommands(cmds, n);
  opacity = opacity < 0 ? 0 : (opacity > 1 ? 1 : opacity);
  if (opacity == 0) return;
  if (!(color[3] > 0 || mode == OverwriteBlend)) return;
  float ps = pixelScale(M);
  std::vector<Polygon> outline =
      strokeShapes(commandsToShapes(cmds, n, false, ps), strokeWidth, cap, join, miterLimit,
                   std::vector<float>(dashes, dashes + nd), ps);
  transformShapes(outline, M);
  float c[4] = {color[0], color[1], color[2], color[3] * opacity};
  fillShapes(img, outline, color_to_rgbx(c), 0, mode);
}

// ---------------------------------------------------------------------------
// Images  images.nim
// ---------------------------------------------------------------------------
// blendRect (draw with an integer translation)  images.nim:468-529
static void blendRect(Image& a, const Image& b, int64_t px, int64_t py, int mode) {
  if (px >= a.width || px + b.width <= 0 || py >= a.height || py + b.height <= 0) {
    if (mode == MaskBlend) fillUnsafe(a, RGBX{0, 0, 0, 0}, 0, a.len());
    return;
  }
  int64_t xStart = std::max<int64_t>(-px, 0), yStart = std::max<int64_t>(-py, 0);
  int64_t xEnd = std::min<int64_t>(b.width, a.width - px), yEnd = std::min<int64_t>(b.height, a.height - py);
  if (mode == MaskBlend) {
    if (yStart + py > 0) fillUnsafe(a, RGBX{0, 0, 0, 0}, 0, (yStart + py) * a.width);
    for (int64_t y = yStart; y < yEnd; y++) {
      if (xStart + px > 0) fillUnsafe(a, RGBX{0, 0, 0, 0}, a.idx(0, y + py), xStart + px);
      RGBX* dl = a.data + a.idx(xStart + px, y + py);
      const RGBX* sl = b.data + b.idx(xStart, y);
      if (g_simd_variant) nl::mask2(dl, sl, xEnd - xStart);
      else for (int64_t i = 0; i < xEnd - xStart; i++) dl[i] = blend_px(MaskBlend, dl[i], sl[i]);
      if (xEnd + px < a.width) fillUnsafe(a, RGBX{0, 0, 0, 0}, a.idx(xEnd + px, y + py), a.width - (xEnd + px));
    }
    if (yEnd + py < a.height)
      fillUnsafe(a, RGBX{0, 0, 0, 0}, a.idx(0, yEnd + py), (a.height - (yEnd + py)) * a.width);
    return;
  }
  for (int64_t y = yStart; y < yEnd; y++) {
    RGBX* dl = a.data + a.idx(xStart + px, y + py);
    const RGBX* sl = b.data + b.idx(xStart, y);
    if (g_simd_variant && mode == NormalBlend) nl::normal2(dl, sl, xEnd - xStart);
    else for (int64_t i = 0; i < xEnd - xStart; i++) dl[i] = blend_px(mode, dl[i], sl[i]);
  }
}

// ---------------------------------------------------------------------------
// draw with a Mat3 transform  images.nim:636-678: the minify/magnify
// pre-passes, then drawSmooth (:531-634) unless the transform is a whole-pixel
// translation (blendRect).  vmath and bumpy are not vendored: Mat3 products,
// the inverse and the line/segment intersection are restated from their
// mathematical definitions (left-to-right sums), pinned by the reference's
// smooth-draw masters.
// ---------------------------------------------------------------------------
static const float kHalf = 0.5f;  // images.nim:5  h

// `mix`(ColorRGBX, ColorRGBX, float32)  common.nim:59-65
static inline RGBX mix_c(RGBX a, RGBX b, float t) {
  const uint32_t x = nim_u32(roundf(t * 255.0f));
  return rgbx((a.r * (255 - x) + b.r * x + 127) / 255, (a.g * (255 - x) + b.g * x + 127) / 255,
              (a.b * (255 - x) + b.b * x + 127) / 255, (a.a * (255 - x) + b.a * x + 127) / 255);
}

// vmath Mat3 * Mat3, column-major: (A B)[c][r] = A[0][r] B[c][0] + A[1][r] B[c][1] + A[2][r] B[c][2]
static Mat3 matmul(const Mat3& A, const Mat3& B) {
  Mat3 R;
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 3; r++)
      R.m[c * 3 + r] = A.m[0 * 3 + r] * B.m[c * 3 + 0] + A.m[1 * 3 + r] * B.m[c * 3 + 1] +
                       A.m[2 * 3 + r] * B.m[c * 3 + 2];
  return R;
}
static Mat3 scale_m(float sx, float sy) { return Mat3{{sx, 0, 0, 0, sy, 0, 0, 0, 1}}; }

// vmath Mat3 inverse: the adjugate over the determinant (cofactor expansion
// along the first column of storage).  a(c, r) = m[c*3 + r].
static Mat3 inverse_m(const Mat3& M) {
  auto a = [&](int c, int r) { return M.m[c * 3 + r]; };
  const float det = a(0, 0) * (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) -
                    a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
                    a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
  const float invDet = 1.0f / det;
  Mat3 R;
  R.m[0] = (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) * invDet;
  R.m[1] = (a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2)) * invDet;
  R.m[2] = (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1)) * invDet;
  R.m[3] = (a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2)) * invDet;
  R.m[4] = (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0)) * invDet;
  R.m[5] = (a(1, 0) * a(0, 2) - a(0, 0) * a(1, 2)) * invDet;
  R.m[6] = (a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1)) * invDet;
  R.m[7] = (a(2, 0) * a(0, 1) - a(0, 0) * a(2, 1)) * invDet;
  R.m[8] = (a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1)) * invDet;
  return R;
}

struct OwnedImage {
  int64_t width = 0, height = 0;
  std::vector<RGBX> px;
  Image view() { return Image{width, height, px.data()}; }
};
static OwnedImage copy_image(const Image& b) {
  OwnedImage o;
  o.width = b.width;
  o.height = b.height;
  o.px.assign(b.data, b.data + b.len());
  return o;
}

// minifyBy2 (power 1)  images.nim:168-232
static OwnedImage minifyBy2(const Image& src) {
  const bool oddW = (src.width % 2) != 0, oddH = (src.height % 2) != 0;
  const int64_t ew = src.width / 2, eh = src.height / 2;
  OwnedImage r;
  r.width = oddW ? ew + 1 : ew;
  r.height = oddH ? eh + 1 : eh;
  r.px.assign((size_t)(r.width * r.height), RGBX{0, 0, 0, 0});
  auto S = [&](int64_t x, int64_t y) { return src.data[src.idx(x, y)]; };
  for (int64_t y = 0; y < eh; y++) {
    for (int64_t x = 0; x < ew; x++) {
      const RGBX a = S(2 * x, 2 * y), b = S(2 * x + 1, 2 * y), c = S(2 * x + 1, 2 * y + 1),
                 d = S(2 * x, 2 * y + 1);
      r.px[(size_t)(r.width * y + x)] =
          rgbx(((uint32_t)a.r + b.r + c.r + d.r + 2) / 4, ((uint32_t)a.g + b.g + c.g + d.g + 2) / 4,
               ((uint32_t)a.b + b.b + c.b + d.b + 2) / 4, ((uint32_t)a.a + b.a + c.a + d.a + 2) / 4);
    }
    if (oddW)
      r.px[(size_t)(r.width * y + r.width - 1)] =
          mul_f(mix_c(S(src.width - 1, 2 * y), S(src.width - 1, 2 * y + 1), 0.5f), 0.5f);
  }
  if (oddH) {
    for (int64_t x = 0; x < ew; x++)
      r.px[(size_t)(r.width * (r.height - 1) + x)] =
          mul_f(mix_c(S(2 * x, src.height - 1), S(2 * x + 1, src.height - 1), 0.5f), 0.5f);
    if (oddW) r.px[(size_t)(r.width * r.height - 1)] = mul_f(S(src.width - 1, src.height - 1), 0.25f);
  }
  return r;
}

// magnifyBy2 (power 1)  images.nim:234-259
static OwnedImage magnifyBy2(const Image& src) {
  OwnedImage r;
  r.width = src.width * 2;
  r.height = src.height * 2;
  r.px.resize((size_t)(r.width * r.height));
  for (int64_t y = 0; y < r.height; y++)
    for (int64_t x = 0; x < r.width; x++) r.px[(size_t)(r.width * y + x)] = src.data[src.idx(x / 2, y / 2)];
  return r;
}

// getRgbaSmooth (not wrapped)  images.nim:367-403; image[x, y] is transparent
// outside the image (:37-40)
static RGBX getRgbaSmooth(const Image& img, float x, float y) {
  const float fx = floorf(x), fy = floorf(y);
  const int64_t x0 = nim_int(fx), y0 = nim_int(fy);
  const int64_t x1 = x0 == INT64_MAX ? x0 : x0 + 1, y1 = y0 == INT64_MAX ? y0 : y0 + 1;
  const float xFractional = x - fx, yFractional = y - fy;
  auto at = [&](int64_t px, int64_t py) {
    return (px >= 0 && px < img.width && py >= 0 && py < img.height) ? img.data[img.idx(px, py)]
                                                                      : RGBX{0, 0, 0, 0};
  };
  const RGBX x0y0 = at(x0, y0), x1y0 = at(x1, y0), x0y1 = at(x0, y1), x1y1 = at(x1, y1);
  RGBX topMix = x0y0;
  if (xFractional > 0 && !same(x0y0, x1y0)) topMix = mix_c(x0y0, x1y0, xFractional);
  RGBX bottomMix = x0y1;
  if (xFractional > 0 && !same(x0y1, x1y1)) bottomMix = mix_c(x0y1, x1y1, xFractional);
  if (yFractional != 0 && !same(topMix, bottomMix)) return mix_c(topMix, bottomMix, yFractional);
  return topMix;
}

// drawSmooth  images.nim:531-634
static void drawSmooth(Image& a, const Image& b, const Mat3& transform, int mode) {
  const Vec2 corners[4] = {mul(transform, v2(0, 0)), mul(transform, v2((float)b.width, 0)),
                           mul(transform, v2((float)b.width, (float)b.height)),
                           mul(transform, v2(0, (float)b.height))};
  const Segment perimeter[4] = {{corners[0], corners[1]}, {corners[1], corners[2]},
                                {corners[2], corners[3]}, {corners[3], corners[0]}};
  const Mat3 inv = inverse_m(transform);
  const Vec2 p = mul(inv, v2(0 + kHalf, 0 + kHalf));
  const Vec2 dx = mul(inv, v2(1 + kHalf, 0 + kHalf)) - p;
  const Vec2 dy = mul(inv, v2(0 + kHalf, 1 + kHalf)) - p;
  int64_t yStart = a.height, yEnd = 0;
  for (const Segment& sg : perimeter) {
    yStart = std::min<int64_t>(yStart, nim_int(floorf(sg.at.y)));
    yEnd = std::max<int64_t>(yEnd, nim_int(ceilf(sg.at.y)));
  }
  yStart = std::clamp<int64_t>(yStart, 0, a.height);
  yEnd = std::clamp<int64_t>(yEnd, 0, a.height);
  const RGBX zero{0, 0, 0, 0};
  if (mode == MaskBlend && yStart > 0) fillUnsafe(a, zero, 0, yStart * a.width);
  for (int64_t y = yStart; y < yEnd; y++) {
    float xMin = (float)a.width, xMax = 0.0f;
    for (float yOffset : {0.0f, 1.0f}) {
      const Vec2 l0 = v2(-1000, (float)y + yOffset), l1 = v2(1000, (float)y + yOffset);
      for (const Segment& sg : perimeter) {
        Vec2 at;
        if (intersectSegLine(sg, l0, l1, at) && sg.to != at) {
          xMin = nmin(xMin, at.x);
          xMax = nmax(xMax, at.x);
        }
      }
    }
    const int64_t xStart = std::clamp<int64_t>(nim_int(floorf(xMin)), 0, a.width);
    const int64_t xEnd = std::clamp<int64_t>(nim_int(ceilf(xMax)), 0, a.width);
    if (xEnd - xStart == 0) continue;
    // a row the perimeter does not cross has xEnd < xStart: its sample loop is
    // empty; MaskBlend still clears [0, xStart) and [xEnd, width), the whole
    // row (OverwriteBlend's copyMem of a negative length, which fails in the
    // reference, copies nothing here)
    Vec2 srcPos = p + dx * (float)xStart + dy * (float)y;
    srcPos = v2(srcPos.x - kHalf, srcPos.y - kHalf);
    RGBX* line = a.data + a.idx(0, y);
    if (mode == MaskBlend && xStart > 0) fillUnsafe(a, zero, a.idx(0, y), xStart);
    for (int64_t x = xStart; x < xEnd; x++) {
      const RGBX s = getRgbaSmooth(b, srcPos.x, srcPos.y);
      srcPos = srcPos + dx;
      line[x] = mode == OverwriteBlend ? s : blend_px(mode, line[x], s);
    }
    if (mode == MaskBlend && a.width - xEnd > 0) fillUnsafe(a, zero, a.idx(xEnd, y), a.width - xEnd);
  }
  if (mode == MaskBlend && a.height - yEnd > 0) fillUnsafe(a, zero, a.idx(0, yEnd), (a.height - yEnd) * a.width);
}

// draw(a, b, transform, blendMode)  images.nim:636-678
static void drawTransform(Image& a, const Image& bIn, Mat3 transform, int mode) {
  const Mat3 inv = inverse_m(transform);
  Vec2 p = mul(inv, v2(0 + kHalf, 0 + kHalf));
  Vec2 dx = mul(inv, v2(1 + kHalf, 0 + kHalf)) - p;
  Vec2 dy = mul(inv, v2(0 + kHalf, 1 + kHalf)) - p;
  float filterBy2 = nmax(length(dx), length(dy));
  // an infinite filterBy2 (a singular transform) would halve forever in the
  // reference's minify loop; raise instead
  if (std::isinf(filterBy2)) throw PixieError("draw transform is not invertible");
  OwnedImage cur = copy_image(bIn);
  while (filterBy2 >= 2.0f) {
    cur = minifyBy2(cur.view());
    p = p / 2;
    dx = dx / 2;
    dy = dy / 2;
    filterBy2 /= 2;
    transform = matmul(transform, scale_m(2, 2));
  }
  while (filterBy2 <= 0.5f) {
    if (cur.width * cur.height > ((int64_t)1 << 30))
      throw PixieError("draw would magnify the source image beyond 2^32 bytes");
    cur = magnifyBy2(cur.view());
    p = p * 2;
    dx = dx * 2;
    dy = dy * 2;
    filterBy2 *= 2;
    transform = matmul(transform, scale_m(1.0f / 2, 1.0f / 2));
  }
  const bool hasRotationOrScaling = !(dx == v2(1, 0) && dy == v2(0, 1));
  const bool smooth = !(length(dx) == 1.0f && length(dy) == 1.0f && fractional(transform.m[6]) == 0.0f &&
                        fractional(transform.m[7]) == 0.0f);
  Image b = cur.view();
  if (hasRotationOrScaling || smooth)
    drawSmooth(a, b, transform, mode);
  else
    blendRect(a, b, nim_i32(transform.m[6]), nim_i32(transform.m[7]), mode);
}

// ---------------------------------------------------------------------------
// Paints  paints.nim, pixie.nim:120-131 (fill with a paint) and fillPath /
// strokePath with a non-solid paint (paths.nim:2115-2142, :2178-2210)
// ---------------------------------------------------------------------------
enum PaintKind {
  SolidPaint = 0, ImagePaint, TiledImagePaint, LinearGradientPaint, RadialGradientPaint, AngularGradientPaint
};
struct ColorStop {
  float color[4];
  float position;
};
struct PaintDesc {
  int kind = SolidPaint;
  int blend = 0;
  float opacity = 1;
  float color[4] = {0, 0, 0, 0};
  Image image{0, 0, nullptr};
  Mat3 imageMat{{1, 0, 0, 0, 1, 0, 0, 0, 1}};
  std::vector<Vec2> handles;
  std::vector<ColorStop> stops;
};

// atan2 for float32 arguments, correctly rounded to float32 (but for inputs
// whose true value lies within ~2^-40 of a rounding boundary): evaluated in
// float-float arithmetic from the mathematics alone, so the CUDA path, which
// runs the same IEEE float32 operations, gets the same floats.  (pixie calls
// the C library's atan2f, which is not reproduced here bit for bit.)

// float-float ("double-float") arithmetic: a value is hi + lo with |lo| <=
// ulp(hi) / 2; two_sum and the fused-multiply-add two_prod give exact error
// terms (Dekker, Knuth), so every operation is a fixed sequence of IEEE
// float32 operations.
struct DF {
  float hi, lo;
};
static inline DF two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return DF{s, (a - (s - bb)) + (b - bb)};
}
static inline DF quick_two_sum(float a, float b) {
  const float s = a + b;
  return DF{s, b - (s - a)};
}
static inline DF two_prod(float a, float b) {
  const float p = a * b;
  return DF{p, std::fma(a, b, -p)};
}
static inline DF df_add(DF x, DF y) {
  DF s = two_sum(x.hi, y.hi);
  const DF t = two_sum(x.lo, y.lo);
  s.lo = s.lo + t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return quick_two_sum(s.hi, s.lo);
}
static inline DF df_neg(DF x) { return DF{-x.hi, -x.lo}; }
static inline DF df_mul(DF x, DF y) {
  DF p = two_prod(x.hi, y.hi);
  p.lo = p.lo + (x.hi * y.lo + x.lo * y.hi);
  return quick_two_sum(p.hi, p.lo);
}
static inline DF df_div(DF x, DF y) {
  const float q1 = x.hi / y.hi;
  DF r = df_add(x, df_neg(df_mul(y, DF{q1, 0.0f})));
  const float q2 = r.hi / y.hi;
  r = df_add(r, df_neg(df_mul(y, DF{q2, 0.0f})));
  const float q3 = r.hi / y.hi;
  return df_add(quick_two_sum(q1, q2), DF{q3, 0.0f});
}
static inline DF df_sqrt(DF a) {  // a > 0
  const float s = std::sqrt(a.hi);
  const DF e = df_add(a, df_neg(two_prod(s, s)));
  return quick_two_sum(s, e.hi / (2.0f * s));
}
#define DF_CONST(v) DF{(float)(v), (float)((v) - (double)(float)(v))}
// atan(x) for x >= 0: pi/2 - atan(1/x) above 1, two halvings
// atan(x) = 2 atan(x / (1 + sqrt(1 + x^2))) to x < 0.2, then 14 Taylor
// terms in Horner form
static inline DF df_atan_unit(DF x) {
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
static inline float atan2_cr(float y, float x) {
  if (std::isnan(x) || std::isnan(y)) return NAN;
  DF r;
  if (y == 0) {
    r = std::signbit(x) ? DF_CONST(3.141592653589793) : DF{0.0f, 0.0f};
  } else if (x == 0) {
    r = DF_CONST(1.5707963267948966);
  } else if (std::isinf(x) || std::isinf(y)) {
    if (std::isinf(x) && std::isinf(y))
      r = x > 0 ? DF_CONST(0.7853981633974483) : DF_CONST(2.356194490192345);
    else if (std::isinf(x))
      r = x > 0 ? DF{0.0f, 0.0f} : DF_CONST(3.141592653589793);
    else
      r = DF_CONST(1.5707963267948966);
  } else {
    const DF q = df_div(DF{std::fabs(y), 0.0f}, DF{std::fabs(x), 0.0f});
    const DF a = df_atan_unit(q);
    r = x > 0 ? a : df_add(DF_CONST(3.141592653589793), df_neg(a));
  }
  const float v = r.hi + r.lo;
  return std::signbit(y) ? -v : v;
}

// chroma mix(Color, Color, t): componentwise lerp a + (b - a) * t
static inline float lerp_f(float a, float b, float t) { return a + (b - a) * t; }

// gradientColor  paints.nim:68-93
static RGBX gradientColor(const PaintDesc& p, float t) {
  int index = -1;
  for (size_t i = 0; i < p.stops.size(); i++) {
    if (p.stops[i].position < t) index = (int)i;
    if (p.stops[i].position > t) break;
  }
  float c[4];
  if (index == -1) {
    memcpy(c, p.stops[0].color, sizeof c);
  } else if (index + 1 >= (int)p.stops.size()) {
    memcpy(c, p.stops[(size_t)index].color, sizeof c);
  } else {
    const ColorStop& a = p.stops[(size_t)index];
    const ColorStop& b = p.stops[(size_t)index + 1];
    const float u = (t - a.position) / (b.position - a.position);
    for (int k = 0; k < 4; k++) c[k] = lerp_f(a.color[k], b.color[k], u);
  }
  c[3] *= p.opacity;
  return color_to_rgbx(c);
}

static bool gradientPrologue(PaintDesc& p, size_t handles, const char* msg) {
  if (p.handles.size() != handles) throw PixieError(msg);
  if (p.stops.empty()) throw PixieError("Gradient must have at least 1 color stop");
  p.opacity = p.opacity < 0 ? 0 : (p.opacity > 1 ? 1 : p.opacity);
  return p.opacity != 0;
}

// fillGradientLinear  paints.nim:95-176.  The horizontal and vertical
// branches fill each column / row with the general formula's value at y = 0
// / x = 0, which equals its value at every y / x (the zero term adds +-0).
static void fillGradientLinear(Image& img, PaintDesc& p) {
  if (!gradientPrologue(p, 2, "Linear gradient requires 2 handles")) return;
  const Vec2 at = p.handles[0], to = p.handles[1];
  const Vec2 d = to - at;
  const float det = d.x * d.x + d.y * d.y;
  for (int64_t y = 0; y < img.height; y++)
    for (int64_t x = 0; x < img.width; x++) {
      const float t = (d.y * ((float)y - at.y) + d.x * ((float)x - at.x)) / det;
      img.data[img.idx(x, y)] = gradientColor(p, t);
    }
}

// vmath rotate(angle): column-major [cos, sin, 0, -sin, cos, 0, 0, 0, 1]
static Mat3 rotate_m(float a) {
  const float sn = sinf(a), cs = cosf(a);
  return Mat3{{cs, sn, 0, -sn, cs, 0, 0, 0, 1}};
}
static Mat3 translate_m(Vec2 v) { return Mat3{{1, 0, 0, 0, 1, 0, v.x, v.y, 1}}; }

// fillGradientRadial  paints.nim:178-205
static void fillGradientRadial(Image& img, PaintDesc& p) {
  if (!gradientPrologue(p, 3, "Radial gradient requires 3 handles")) return;
  const Vec2 center = p.handles[0], edge = p.handles[1], skew = p.handles[2];
  const float distanceX = length(center - edge), distanceY = length(center - skew);
  const float gradientAngle = fixAngle(angleOf(normalize(center - edge)));
  const Mat3 mat = inverse_m(matmul(matmul(translate_m(center), rotate_m(gradientAngle)),
                                    scale_m(distanceX, distanceY)));
  for (int64_t y = 0; y < img.height; y++)
    for (int64_t x = 0; x < img.width; x++) {
      const float t = length(mul(mat, v2((float)x, (float)y)));
      img.data[img.idx(x, y)] = gradientColor(p, t);
    }
}

// fillGradientAngular  paints.nim:207-229 (its error text says "2 handles")
static void fillGradientAngular(Image& img, PaintDesc& p) {
  if (!gradientPrologue(p, 3, "Angular gradient requires 2 handles")) return;
  const Vec2 center = p.handles[0], edge = p.handles[1];
  const float f32PI = (float)kPI;
  const float gradientAngle = fixAngle(angleOf(normalize(edge - center)));
  for (int64_t y = 0; y < img.height; y++)
    for (int64_t x = 0; x < img.width; x++) {
      const Vec2 v = normalize(v2((float)x, (float)y) - center);
      const float angle = atan2_cr(v.y, v.x);
      const float t = fixAngle(angle + gradientAngle + f32PI / 2) / 2 / f32PI + 0.5f;
      img.data[img.idx(x, y)] = gradientColor(p, t);
    }
}

static void fillGradient(Image& img, PaintDesc p) {  // paints.nim:231-241
  switch (p.kind) {
    case LinearGradientPaint: fillGradientLinear(img, p); break;
    case RadialGradientPaint: fillGradientRadial(img, p); break;
    case AngularGradientPaint: fillGradientAngular(img, p); break;
    default: throw PixieError("Paint must be a gradient");
  }
}

// applyOpacity  images.nim:261-277
static void applyOpacity(Image& img, float opacity) {
  const uint32_t o = (uint16_t)nim_i32(roundf(255 * opacity));
  if (o == 255) return;
  if (o == 0) {
    fillUnsafe(img, RGBX{0, 0, 0, 0}, 0, img.len());
    return;
  }
  for (int64_t i = 0; i < img.len(); i++) {
    RGBX& c = img.data[i];
    c = rgbx((c.r * o) / 255, (c.g * o) / 255, (c.b * o) / 255, (c.a * o) / 255);
  }
}

// getRgbaSmooth with wrapped = true (images.nim:381-385): the taps are
// image.unsafe[x mod w, y mod h] with Nim's truncating mod, so a negative
// coordinate addresses data[w * (y mod h) + (x mod w)] linearly (the previous
// row's last pixel for x = -1); an address outside the buffer, which reads
// foreign memory in the reference, reads transparent here.
static RGBX getRgbaSmoothWrapped(const Image& img, float x, float y) {
  const float fx = floorf(x), fy = floorf(y);
  const int64_t x0 = nim_int(fx), y0 = nim_int(fy);
  const int64_t x1 = x0 == INT64_MAX ? x0 : x0 + 1, y1 = y0 == INT64_MAX ? y0 : y0 + 1;
  const float xFractional = x - fx, yFractional = y - fy;
  auto at = [&](int64_t px, int64_t py) {
    const int64_t i = img.width * (py % img.height) + (px % img.width);
    return (i >= 0 && i < img.len()) ? img.data[i] : RGBX{0, 0, 0, 0};
  };
  const RGBX x0y0 = at(x0, y0), x1y0 = at(x1, y0), x0y1 = at(x0, y1), x1y1 = at(x1, y1);
  RGBX topMix = x0y0;
  if (xFractional > 0 && !same(x0y0, x1y0)) topMix = mix_c(x0y0, x1y0, xFractional);
  RGBX bottomMix = x0y1;
  if (xFractional > 0 && !same(x0y1, x1y1)) bottomMix = mix_c(x0y1, x1y1, xFractional);
  if (yFractional != 0 && !same(topMix, bottomMix)) return mix_c(topMix, bottomMix, yFractional);
  return topMix;
}

// drawCorrect  images.nim:405-445 (drawTiled :680-683 is tiled = true): every
// destination pixel samples inverseTransform * (x + h, y + h) - h
static void drawCorrect(Image& a, const Image& bIn, const Mat3& transform, int mode, bool tiled) {
  Mat3 inv = inverse_m(transform);
  Vec2 p = mul(inv, v2(0 + kHalf, 0 + kHalf));
  Vec2 dx = mul(inv, v2(1 + kHalf, 0 + kHalf)) - p;
  Vec2 dy = mul(inv, v2(0 + kHalf, 1 + kHalf)) - p;
  float filterBy2 = nmax(length(dx), length(dy));
  if (std::isinf(filterBy2)) throw PixieError("draw transform is not invertible");
  OwnedImage cur = copy_image(bIn);
  while (filterBy2 >= 2.0f) {
    cur = minifyBy2(cur.view());
    p = p / 2;
    dx = dx / 2;
    dy = dy / 2;
    filterBy2 /= 2;
    inv = matmul(scale_m(0.5f, 0.5f), inv);
  }
  while (filterBy2 <= 0.5f) {
    if (cur.width * cur.height > ((int64_t)1 << 30))
      throw PixieError("draw would magnify the source image beyond 2^32 bytes");
    cur = magnifyBy2(cur.view());
    p = p * 2;
    dx = dx * 2;
    dy = dy * 2;
    filterBy2 *= 2;
    inv = matmul(scale_m(2, 2), inv);
  }
  const Image b = cur.view();
  for (int64_t y = 0; y < a.height; y++)
    for (int64_t x = 0; x < a.width; x++) {
      const Vec2 sp = mul(inv, v2((float)x + kHalf, (float)y + kHalf));
      const float xf = sp.x - kHalf, yf = sp.y - kHalf;
      const RGBX s = tiled ? getRgbaSmoothWrapped(b, xf, yf) : getRgbaSmooth(b, xf, yf);
      RGBX& d = a.data[a.idx(x, y)];
      d = blend_px(mode, d, s);
    }
}

// the paint image of a non-solid paint (paths.nim:2121-2134): the image
// paint drawn, tiled, or the gradient, with the paint at opacity 1
static void paintImage(Image& fill, const PaintDesc& paint) {
  PaintDesc p = paint;
  p.opacity = 1;
  switch (p.kind) {
    case ImagePaint: drawTransform(fill, p.image, p.imageMat, NormalBlend); break;
    case TiledImagePaint: drawCorrect(fill, p.image, p.imageMat, NormalBlend, true); break;
    default: fillGradient(fill, p); break;
  }
}
// mask -> fill -> MaskBlend -> draw  paths.nim:2115-2142
static void compositePaint(Image& img, Image& mask, const PaintDesc& paint) {
  OwnedImage fill;
  fill.width = img.width;
  fill.height = img.height;
  fill.px.assign((size_t)img.len(), RGBX{0, 0, 0, 0});
  Image F = fill.view();
  paintImage(F, paint);
  const float op = paint.opacity < 0 ? 0 : (paint.opacity > 1 ? 1 : paint.opacity);
  if (op != 1) applyOpacity(mask, op);
  blendRect(F, mask, 0, 0, MaskBlend);
  blendRect(img, F, 0, 0, paint.blend);
}

static void fillPathPaint(Image& img, const float* cmds, int64_t n, const PaintDesc& paint, const Mat3& M,
                          int rule) {
  const float op = paint.opacity < 0 ? 0 : (paint.opacity > 1 ? 1 : paint.opacity);
  if (op == 0) return;
  if (paint.kind == SolidPaint) {
    fillPath(img, cmds, n, paint.color, op, paint.blend, M, rule);
    return;
  }
  validateCommands(cmds, n);
  OwnedImage mask;
  mask.width = img.width;
  mask.height = img.height;
  mask.px.assign((size_t)img.len(), RGBX{0, 0, 0, 0});
  Image Mk = mask.view();
  const float white[4] = {1, 1, 1, 1};
  fillPath(Mk, cmds, n, white, 1, NormalBlend, M, rule);
  compositePaint(img, Mk, paint);
}

static void strokePathPaint(Image& img, const float* cmds, int64_t n, const PaintDesc& paint, const Mat3& M,
                            float width, int cap, int join, float miter, const float* dashes, int nd) {
  const float op = paint.opacity < 0 ? 0 : (paint.opacity > 1 ? 1 : paint.opacity);
  if (op == 0) return;
  if (paint.kind == SolidPaint) {
    strokePath(img, cmds, n, paint.color, op, paint.blend, M, width, cap, join, miter, dashes, nd);
    return;
  }
  validateCommands(cmds, n);
  OwnedImage mask;
  mask.width = img.width;
  mask.height = img.height;
  mask.px.assign((size_t)img.len(), RGBX{0, 0, 0, 0});
  Image Mk = mask.view();
  const float white[4] = {1, 1, 1, 1};
  strokePath(Mk, cmds, n, white, 1, NormalBlend, M, width, cap, join, miter, dashes, nd);
  compositePaint(img, Mk, paint);
}

// fill(image, paint)  pixie.nim:120-131
static void fillWithPaint(Image& img, const PaintDesc& paint) {
  switch (paint.kind) {
    case SolidPaint: fillUnsafe(img, color_to_rgbx(paint.color), 0, img.len()); break;
    case ImagePaint:
    case TiledImagePaint: {
      fillUnsafe(img, RGBX{0, 0, 0, 0}, 0, img.len());
      const float rect[] = {Move, 0, 0, Line, (float)img.width, 0, Line, (float)img.width, (float)img.height,
                            Line, 0, (float)img.height, Close};
      fillPathPaint(img, rect, (int64_t)(sizeof rect / sizeof rect[0]), paint, Mat3{{1, 0, 0, 0, 1, 0, 0, 0, 1}},
                    0);
      break;
    }
    default: fillGradient(img, paint); break;
  }
}

// gaussianKernel  internal.nim:17-34.  `s` and the exp() argument are float32;
// `1 / sqrt(2 * PI * s^2) * exp(...)` meets the float64 constant PI and is
// float64; `total` is a float64 variable and
// `floats[i] / total` divides in float64.
static std::vector<uint16_t> gaussianKernel(int64_t radius) {
  size_t n = (size_t)(radius * 2 + 1);
  std::vector<uint16_t> out(n);
  std::vector<float> floats(n);
  double total = 0.0;
  for (int64_t step = -radius; step <= radius; step++) {
    float s = (float)radius / 2.2f;
    float e = expf((-1.0f * ((float)step * (float)step)) / (2.0f * (s * s)));
    double a64 = 1.0 / sqrt((2 * kPI) * (double)(s * s)) * (double)e;
    float a = (float)a64;
    floats[(size_t)(step + radius)] = a;
    total += a64;
  }
  for (size_t i = 0; i < n; i++) floats[i] = (float)((double)floats[i] / total);
  for (size_t i = 0; i < n; i++) out[i] = nim_u16(roundf(floats[i] * 255 * 256));
  return out;
}

static void blur(Image& img, float radiusF, RGBX oob) {  // images.nim:304-365
  int64_t radius = nim_int(roundf(radiusF));
  if (radius == 0) return;
  if (radius < 0) throw PixieError("Cannot apply negative blur");
  std::vector<uint16_t> kernel = gaussianKernel(radius);
  const int64_t W = img.width, H = img.height;
  std::vector<RGBX> blurX((size_t)(W * H));  // transposed: H wide, W tall
  auto acc = [](uint32_t v[4], RGBX p, uint32_t k) {
    v[0] += p.r * k;
    v[1] += p.g * k;
    v[2] += p.b * k;
    v[3] += p.a * k;
  };
  auto out = [](const uint32_t v[4]) { return rgbx(v[0] / 256 / 255, v[1] / 256 / 255, v[2] / 256 / 255, v[3] / 256 / 255); };
  for (int64_t y = 0; y < H; y++)
    for (int64_t x = 0; x < W; x++) {
      uint32_t v[4] = {0, 0, 0, 0};
      for (int64_t xx = x - radius; xx < std::min<int64_t>(x + radius, 0); xx++) acc(v, oob, kernel[(size_t)(xx - x + radius)]);
      for (int64_t xx = std::max<int64_t>(x - radius, 0); xx <= std::min<int64_t>(x + radius, W - 1); xx++)
        acc(v, img.data[img.idx(xx, y)], kernel[(size_t)(xx - x + radius)]);
      for (int64_t xx = std::max<int64_t>(x - radius, W); xx <= x + radius; xx++) acc(v, oob, kernel[(size_t)(xx - x + radius)]);
      blurX[(size_t)(H * x + y)] = out(v);
    }
  for (int64_t y = 0; y < H; y++)
    for (int64_t x = 0; x < W; x++) {
      uint32_t v[4] = {0, 0, 0, 0};
      for (int64_t yy = y - radius; yy < std::min<int64_t>(y + radius, 0); yy++) acc(v, oob, kernel[(size_t)(yy - y + radius)]);
      for (int64_t yy = std::max<int64_t>(y - radius, 0); yy <= std::min<int64_t>(y + radius, H - 1); yy++)
        acc(v, blurX[(size_t)(H * x + yy)], kernel[(size_t)(yy - y + radius)]);
      for (int64_t yy = std::max<int64_t>(y - radius, H); yy <= y + radius; yy++) acc(v, oob, kernel[(size_t)(yy - y + radius)]);
      img.data[img.idx(x, y)] = out(v);
    }
}

static void spread(Image& img, float spreadF) {  // images.nim:700-758
  int64_t sp = nim_int(roundf(spreadF));
  if (sp == 0) return;
  const int64_t W = img.width, H = img.height;
  std::vector<uint8_t> sx((size_t)(W * H));  // transposed alpha
  if (sp > 0) {
    for (int64_t y = 0; y < H; y++)
      for (int64_t x = 0; x < W; x++) {
        uint8_t mv = 0;
        for (int64_t xx = std::max<int64_t>(x - sp, 0); xx <= std::min<int64_t>(x + sp, W - 1); xx++) {
          uint8_t v = img.data[img.idx(xx, y)].a;
          if (v > mv) mv = v;
          if (mv == 255) break;
        }
        sx[(size_t)(H * x + y)] = mv;
      }
    for (int64_t y = 0; y < H; y++)
      for (int64_t x = 0; x < W; x++) {
        uint8_t mv = 0;
        for (int64_t yy = std::max<int64_t>(y - sp, 0); yy <= std::min<int64_t>(y + sp, H - 1); yy++) {
          uint8_t v = sx[(size_t)(H * x + yy)];
          if (v > mv) mv = v;
          if (mv == 255) break;
        }
        img.data[img.idx(x, y)] = RGBX{0, 0, 0, mv};
      }
  } else {
    sp = -sp;
    for (int64_t y = 0; y < H; y++)
      for (int64_t x = 0; x < W; x++) {
        uint8_t mv = 255;
        for (int64_t xx = std::max<int64_t>(x - sp, 0); xx <= std::min<int64_t>(x + sp, W - 1); xx++) {
          uint8_t v = img.data[img.idx(xx, y)].a;
          if (v < mv) mv = v;
          if (mv == 0) break;
        }
        sx[(size_t)(H * x + y)] = mv;
      }
    for (int64_t y = 0; y < H; y++)
      for (int64_t x = 0; x < W; x++) {
        uint8_t mv = 255;
        for (int64_t yy = std::max<int64_t>(y - sp, 0); yy <= std::min<int64_t>(y + sp, H - 1); yy++) {
          uint8_t v = sx[(size_t)(H * x + yy)];
          if (v < mv) mv = v;
          if (mv == 0) break;
        }
        img.data[img.idx(x, y)] = RGBX{0, 0, 0, mv};
      }
  }
}

}  // namespace pxo

// ===========================================================================
// C interface for the Python test harness (ctypes)
// ===========================================================================
using namespace pxo;

static thread_local std::string g_err;
static int fail(const std::exception& e) {
  g_err = e.what();
  return 1;
}
static Mat3 mat_from(const float* m) {
  Mat3 M;
  static const float I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  memcpy(M.m, m ? m : I, sizeof M.m);
  return M;
}

extern "C" {

const char* pxo_last_error(void) { return g_err.c_str(); }

// Golden-pinning mode switch (see g_golden_mode); 0 = scalar oracle.
void pxo_set_golden_mode(int on) { g_golden_mode = on; }

// The C library's sinf / cosf (what the reference's float32 sin/cos call),
// element-wise, for the arc-flattening gate test.
void pxo_libm_sincosf(const float* x, int64_t n, float* s, float* c) {
  for (int64_t i = 0; i < n; i++) {
    s[i] = sinf(x[i]);
    c[i] = cosf(x[i]);
  }
}

// The C library's atan2f and the shared float-float arctangent, element-wise
// (for comparing the stroke joins' decisions under both).
void pxo_atan2_pairs(const float* y, const float* x, int64_t n, float* libm, float* cr) {
  for (int64_t i = 0; i < n; i++) {
    libm[i] = atan2f(y[i], x[i]);
    cr[i] = atan2_cr(y[i], x[i]);
  }
}

// applyOpacity  images.nim:261-277
int pxo_apply_opacity(uint8_t* rgbx_data, int64_t w, int64_t h, float opacity) {
  Image img{w, h, (RGBX*)rgbx_data};
  applyOpacity(img, opacity);
  return 0;
}

// 1: the NEON line kernels of the timed CPU baseline (see nl::), 0: scalar.
void pxo_set_simd_variant(int on) { g_simd_variant = on; }

// This thread's row window for fills and strokes (see g_row_lo).
void pxo_set_row_window(int64_t lo, int64_t hi) {
  g_row_lo = lo;
  g_row_hi = hi;
}

int pxo_fill_path(uint8_t* rgbx_data, int64_t w, int64_t h, const float* cmds, int64_t n,
                  const float* color, float opacity, int blend, const float* mat, int rule) {
  try {
    Image img{w, h, (RGBX*)rgbx_data};
    fillPath(img, cmds, n, color, opacity, blend, mat_from(mat), rule);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int pxo_stroke_path(uint8_t* rgbx_data, int64_t w, int64_t h, const float* cmds, int64_t n,
                    const float* color, float opacity, int blend, const float* mat, float width,
                    int cap, int join, float miterLimit, const float* dashes, int nd) {
  try {
    Image img{w, h, (RGBX*)rgbx_data};
    strokePath(img, cmds, n, color, opacity, blend, mat_from(mat), width, cap, join, miterLimit,
               dashes, nd);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

// Flattened polygons of a fill (commandsToShapes + transform), for
// cross-checking the product's flattening.  Writes up to cap points and the
// per-polygon point counts; returns the number of polygons or -1.
int64_t pxo_shapes(const float* cmds, int64_t n, const float* mat, int closeSubpaths, float* pts,
                   int64_t cap, int64_t* counts, int64_t countCap, int64_t* totalPts) {
  try {
    validateCommands(cmds, n);
    Mat3 M = mat_from(mat);
    auto shapes = commandsToShapes(cmds, n, closeSubpaths != 0, pixelScale(M));
    transformShapes(shapes, M);
    int64_t k = 0;
    for (size_t s = 0; s < shapes.size(); s++) {
      if ((int64_t)s < countCap) counts[s] = (int64_t)shapes[s].size();
      for (auto& v : shapes[s]) {
        if (k < cap) {
          pts[2 * k] = v.x;
          pts[2 * k + 1] = v.y;
        }
        k++;
      }
    }
    *totalPts = k;
    return (int64_t)shapes.size();
  } catch (const std::exception& e) {
    fail(e);
    return -1;
  }
}

// Stroke outline polygons (before the transform), for cross-checking.
int64_t pxo_stroke_shapes(const float* cmds, int64_t n, const float* mat, float width, int cap,
                          int join, float miterLimit, const float* dashes, int nd, float* pts,
                          int64_t ptCap, int64_t* counts, int64_t countCap, int64_t* totalPts) {
  try {
    validateCommands(cmds, n);
    Mat3 M = mat_from(mat);
    float ps = pixelScale(M);
    auto shapes = strokeShapes(commandsToShapes(cmds, n, false, ps), width, cap, join, miterLimit,
                               std::vector<float>(dashes, dashes + nd), ps);
    int64_t k = 0;
    for (size_t s = 0; s < shapes.size(); s++) {
      if ((int64_t)s < countCap) counts[s] = (int64_t)shapes[s].size();
      for (auto& v : shapes[s]) {
        if (k < ptCap) {
          pts[2 * k] = v.x;
          pts[2 * k + 1] = v.y;
        }
        k++;
      }
    }
    *totalPts = k;
    return (int64_t)shapes.size();
  } catch (const std::exception& e) {
    fail(e);
    return -1;
  }
}

int pxo_draw(uint8_t* a, int64_t aw, int64_t ah, const uint8_t* b, int64_t bw, int64_t bh,
             int64_t tx, int64_t ty, int blend) {
  try {
    Image A{aw, ah, (RGBX*)a};
    Image B{bw, bh, (RGBX*)b};
    blendRect(A, B, tx, ty, blend);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

// A paint as floats: [kind, blend, opacity, r, g, b, a, imageMat[9],
// nHandles, x, y, ..., nStops, r, g, b, a, position, ...]; the image of an
// image paint is passed beside it.
static PaintDesc paint_from(const float* f, int64_t nf, const uint8_t* img, int64_t iw, int64_t ih) {
  PaintDesc p;
  if (nf < 18) throw PixieError("bad paint encoding");
  p.kind = (int)f[0];
  p.blend = (int)f[1];
  p.opacity = f[2];
  memcpy(p.color, f + 3, sizeof p.color);
  memcpy(p.imageMat.m, f + 7, sizeof p.imageMat.m);
  int64_t k = 16;
  const int64_t nh = (int64_t)f[k++];
  if (k + 2 * nh + 1 > nf) throw PixieError("bad paint encoding");
  for (int64_t i = 0; i < nh; i++, k += 2) p.handles.push_back(v2(f[k], f[k + 1]));
  const int64_t ns = (int64_t)f[k++];
  if (k + 5 * ns > nf) throw PixieError("bad paint encoding");
  for (int64_t i = 0; i < ns; i++, k += 5) {
    ColorStop c;
    memcpy(c.color, f + k, sizeof c.color);
    c.position = f[k + 4];
    p.stops.push_back(c);
  }
  p.image = Image{iw, ih, (RGBX*)img};
  if ((p.kind == ImagePaint || p.kind == TiledImagePaint) && (!img || iw <= 0 || ih <= 0))
    throw PixieError("Image paint needs an image");
  return p;
}

int pxo_fill_path_paint(uint8_t* rgbx_data, int64_t w, int64_t h, const float* cmds, int64_t n,
                        const float* paint, int64_t np, const uint8_t* pimg, int64_t pw, int64_t ph,
                        const float* mat, int rule) {
  try {
    Image img{w, h, (RGBX*)rgbx_data};
    fillPathPaint(img, cmds, n, paint_from(paint, np, pimg, pw, ph), mat_from(mat), rule);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int pxo_stroke_path_paint(uint8_t* rgbx_data, int64_t w, int64_t h, const float* cmds, int64_t n,
                          const float* paint, int64_t np, const uint8_t* pimg, int64_t pw, int64_t ph,
                          const float* mat, float width, int cap, int join, float miter, const float* dashes,
                          int nd) {
  try {
    Image img{w, h, (RGBX*)rgbx_data};
    strokePathPaint(img, cmds, n, paint_from(paint, np, pimg, pw, ph), mat_from(mat), width, cap, join, miter,
                    dashes, nd);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int pxo_fill_paint(uint8_t* rgbx_data, int64_t w, int64_t h, const float* paint, int64_t np, const uint8_t* pimg,
                   int64_t pw, int64_t ph) {
  try {
    Image img{w, h, (RGBX*)rgbx_data};
    fillWithPaint(img, paint_from(paint, np, pimg, pw, ph));
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

float pxo_atan2(float y, float x) { return atan2_cr(y, x); }

int pxo_draw_tiled(uint8_t* a, int64_t aw, int64_t ah, const uint8_t* b, int64_t bw, int64_t bh,
                   const float* mat3, int blend) {
  try {
    Image A{aw, ah, (RGBX*)a};
    Image B{bw, bh, (RGBX*)b};
    Mat3 M;
    memcpy(M.m, mat3, sizeof(M.m));
    drawCorrect(A, B, M, blend, true);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int pxo_draw_transform(uint8_t* a, int64_t aw, int64_t ah, const uint8_t* b, int64_t bw, int64_t bh,
                       const float* mat3, int blend) {
  try {
    Image A{aw, ah, (RGBX*)a};
    Image B{bw, bh, (RGBX*)b};
    Mat3 M;
    memcpy(M.m, mat3, sizeof(M.m));
    drawTransform(A, B, M, blend);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

// minifyBy2 / magnifyBy2 with power 1 into a caller buffer of the result size
int pxo_minify_by2(const uint8_t* src, int64_t w, int64_t h, uint8_t* out) {
  OwnedImage r = minifyBy2(Image{w, h, (RGBX*)src});
  memcpy(out, r.px.data(), r.px.size() * 4);
  return 0;
}
int pxo_magnify_by2(const uint8_t* src, int64_t w, int64_t h, uint8_t* out) {
  OwnedImage r = magnifyBy2(Image{w, h, (RGBX*)src});
  memcpy(out, r.px.data(), r.px.size() * 4);
  return 0;
}

int pxo_blend_pixels(int blend, const uint8_t* backdrop, const uint8_t* source, uint8_t* out,
                     int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    RGBX b, s;
    memcpy(&b, backdrop + 4 * i, 4);
    memcpy(&s, source + 4 * i, 4);
    RGBX r = blend_px(blend, b, s);
    memcpy(out + 4 * i, &r, 4);
  }
  return 0;
}

int pxo_fill(uint8_t* rgbx_data, int64_t w, int64_t h, const float* color) {
  Image img{w, h, (RGBX*)rgbx_data};
  fillUnsafe(img, color_to_rgbx(color), 0, img.len());
  return 0;
}

int pxo_color_to_rgbx(const float* color, uint8_t* out) {
  RGBX r = color_to_rgbx(color);
  memcpy(out, &r, 4);
  return 0;
}

int pxo_blur(uint8_t* rgbx_data, int64_t w, int64_t h, float radius, const uint8_t* oob) {
  try {
    Image img{w, h, (RGBX*)rgbx_data};
    RGBX o;
    memcpy(&o, oob, 4);
    blur(img, radius, o);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int pxo_gaussian_kernel(int64_t radius, uint16_t* out) {
  auto k = gaussianKernel(radius);
  memcpy(out, k.data(), k.size() * 2);
  return (int)k.size();
}

int pxo_spread(uint8_t* rgbx_data, int64_t w, int64_t h, float sp) {
  Image img{w, h, (RGBX*)rgbx_data};
  spread(img, sp);
  return 0;
}

// shadow  images.nim:760-776 (integer offsets: the blendRect branch of draw)
int pxo_shadow(const uint8_t* src, int64_t w, int64_t h, int64_t ox, int64_t oy, float sp,
               float blurR, const float* color, uint8_t* out) {
  try {
    std::vector<RGBX> mask((size_t)(w * h));
    Image M{w, h, mask.data()};
    Image S{w, h, (RGBX*)src};
    if (ox == 0 && oy == 0) {
      memcpy(mask.data(), src, (size_t)(w * h * 4));
    } else {
      blendRect(M, S, ox, oy, OverwriteBlend);
    }
    spread(M, sp);
    blur(M, blurR, RGBX{0, 0, 0, 0});
    Image R{w, h, (RGBX*)out};
    fillUnsafe(R, color_to_rgbx(color), 0, R.len());
    blendRect(R, M, 0, 0, MaskBlend);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

// shadow with any offset: draw(image, translate(offset), OverwriteBlend) takes
// drawSmooth for a fractional offset (images.nim:760-769, :636-678)
int pxo_shadow_f(const uint8_t* src, int64_t w, int64_t h, float ox, float oy, float sp, float blurR,
                 const float* color, uint8_t* out) {
  try {
    std::vector<RGBX> mask((size_t)(w * h), RGBX{0, 0, 0, 0});
    Image M{w, h, mask.data()};
    Image S{w, h, (RGBX*)src};
    if (ox == 0 && oy == 0)
      memcpy(mask.data(), src, (size_t)(w * h * 4));
    else
      drawTransform(M, S, translate_m(v2(ox, oy)), OverwriteBlend);
    spread(M, sp);
    blur(M, blurR, RGBX{0, 0, 0, 0});
    Image R{w, h, (RGBX*)out};
    fillUnsafe(R, color_to_rgbx(color), 0, R.len());
    blendRect(R, M, 0, 0, MaskBlend);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

// toStraightAlpha over a buffer (internal.nim:76-84), for comparing with the
// straight-alpha golden PNGs.
int pxo_to_straight(uint8_t* rgbx_data, int64_t npx) {
  init_straight();
  for (int64_t i = 0; i < npx; i++) {
    uint8_t* p = rgbx_data + 4 * i;
    uint8_t a = p[3];
    p[0] = g_straight[a][p[0]];
    p[1] = g_straight[a][p[1]];
    p[2] = g_straight[a][p[2]];
  }
  return 0;
}

}  // extern "C"
