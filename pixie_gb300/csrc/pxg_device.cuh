// Device-side scalar semantics shared by every kernel: pixie's premultiplied
// RGBX pixel, its integer blend modes (src/pixie/blends.nim), its colour
// multiplies (src/pixie/common.nim:67-90) and Nim's float->int conversions.
// Compiled with -fmad=false so float32 expressions keep the reference's
// operation order and rounding.
#pragma once
#include <cstdint>
#include <initializer_list>
#include <utility>

#include <cuda_runtime.h>

namespace pxg {

enum Blend {
  kNormal = 0, kDarken, kMultiply, kColorBurn, kLighten, kScreen, kColorDodge, kOverlay,
  kSoftLight, kHardLight, kDifference, kExclusion, kHue, kSaturation, kColor, kLuminosity,
  kMask, kOverwrite, kSubtractMask, kExcludeMask, kNumBlends
};

struct Px {
  uint32_t r, g, b, a;
};
__device__ __forceinline__ Px unpack(uint32_t v) {
  return Px{v & 255u, (v >> 8) & 255u, (v >> 16) & 255u, v >> 24};
}
__device__ __forceinline__ uint32_t pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
  return (r & 255u) | ((g & 255u) << 8) | ((b & 255u) << 16) | ((a & 255u) << 24);
}

// Programmatic dependent launch: a kernel launched with launch_pdl lets the
// next PDL kernel on its stream be set up while its own blocks finish
// (pdl_trigger), and waits before touching memory until the kernel before
// it has completed with its writes visible (pdl_wait).  Both are no-ops for
// an ordinary launch.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// A kernel that may be launched late waits at its start (late = 0) or just
// before it exits (late = 1).  It lets the next kernel be set up only once
// its own start-wait has passed: a kernel launched after one that waits at
// its start then never overlaps a kernel still running before that one (the
// in-flight set dep_late checks against restarts there).
__device__ __forceinline__ void pdl_late_entry(int late) {
  if (!late) pdl_wait();
  pdl_trigger();
}
__device__ __forceinline__ void pdl_late_exit(int late) {
  if (late) pdl_wait();
}
// A device buffer a kernel reads or writes.
struct Span {
  const void* p;
  size_t n;
};
// Whether the kernel about to be launched on st may run without waiting for
// the kernel before it (and wait only before it exits): true when its
// buffers are disjoint from those of every kernel that may still be running.
// Records them; the launch's note_launch follows.  Defined in composite.cu.
bool dep_late(cudaStream_t st, std::initializer_list<Span> writes, std::initializer_list<Span> reads);
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Nim float32 -> int conversions as the reference's x86-64 builds perform them
// (cvttss2si: NaN and out-of-range give INT_MIN).
__device__ __forceinline__ long long nim_int(float f) {
  if (!(f >= -9223372036854775808.0f && f < 9223372036854775808.0f)) return (long long)(-9223372036854775807LL - 1);
  return (long long)f;
}
__device__ __forceinline__ int nim_i32(float f) {
  if (!(f >= -2147483648.0f && f < 2147483648.0f)) return (int)0x80000000u;
  return (int)f;
}
__device__ __forceinline__ uint32_t nim_u32(float f) { return (uint32_t)(unsigned long long)nim_int(f); }
__device__ __forceinline__ float nmin(float x, float y) { return x <= y ? x : y; }
__device__ __forceinline__ float nmax(float x, float y) { return y <= x ? x : y; }

// Two channels per 32-bit word: bytes 0 and 2 (r, b) or, after >> 8, bytes 1
// and 3 (g, a), each in its own 16-bit lane.  floor(x / 255) of both lanes at
// once is (x + 1 + (x >> 8)) >> 8 -- exact for every 0 <= x <= 65534, checked
// exhaustively -- and no lane carries into the other (x + 1 + 254 < 2^16).
__device__ __forceinline__ uint32_t div255_lanes(uint32_t x) {
  return ((x + 0x00010001u + ((x >> 8) & 0x00FF00FFu)) >> 8) & 0x00FF00FFu;
}
// floor(c * k / 255) of all four channels of c (k <= 255)
__device__ __forceinline__ uint32_t mul_div255_px(uint32_t c, uint32_t k) {
  return div255_lanes((c & 0x00FF00FFu) * k) | (div255_lanes(((c >> 8) & 0x00FF00FFu) * k) << 8);
}

// `*`(ColorRGBX, uint8)  common.nim:79-90: (c * k + 127) div 255 per channel
__device__ __forceinline__ uint32_t mul_c(uint32_t c, uint32_t k) {
  if (k == 0) return 0u;
  if (k == 255) return c;
  return div255_lanes((c & 0x00FF00FFu) * k + 0x007F007Fu) |
         (div255_lanes(((c >> 8) & 0x00FF00FFu) * k + 0x007F007Fu) << 8);
}
// `*`(ColorRGBX, float32)  common.nim:67-77
__device__ __forceinline__ uint32_t mul_f(uint32_t c, float opacity) {
  if (opacity == 0.0f) return 0u;
  uint32_t x = nim_u32(roundf(opacity * 255.0f));
  Px p = unpack(c);
  return pack((p.r * x + 127) / 255, (p.g * x + 127) / 255, (p.b * x + 127) / 255,
              (p.a * x + 127) / 255);
}

__device__ __forceinline__ uint32_t blendAlpha(uint32_t b, uint32_t s) {  // blends.nim:41-43
  return (s + ((b * (255 - s)) / 255)) & 255u;
}
__device__ __forceinline__ uint32_t screen1(uint32_t b, uint32_t s) {  // :45-46
  return (uint32_t)((int)(b + s) - (int)((b * s) / 255)) & 255u;
}
__device__ __forceinline__ uint32_t hardLight1(uint32_t bc, uint32_t ba, uint32_t sc, uint32_t sa) {
  if (sc * 2 <= sa) return ((2 * sc * bc + sc * (255 - ba) + bc * (255 - sa)) / 255) & 255u;
  return screen1(bc, sc);
}

// blendNormal  blends.nim:60-70: source + backdrop * (255 - sa) div 255 on
// every channel (blendAlpha is the same expression on alpha), uint8 wrap-around
// on the sum; two channels per word (div255_lanes)
__device__ __forceinline__ uint32_t blendNormal(uint32_t bv, uint32_t sv) {
  const uint32_t sa = sv >> 24, ba = bv >> 24;
  if (ba == 0 || sa == 255) return sv;
  if (sa == 0) return bv;
  const uint32_t k = 255 - sa;
  const uint32_t rb = (div255_lanes((bv & 0x00FF00FFu) * k) + (sv & 0x00FF00FFu)) & 0x00FF00FFu;
  const uint32_t ga = (div255_lanes(((bv >> 8) & 0x00FF00FFu) * k) + ((sv >> 8) & 0x00FF00FFu)) & 0x00FF00FFu;
  return rb | (ga << 8);
}
__device__ __forceinline__ uint32_t blendMaskPx(uint32_t bv, uint32_t sv) {  // :227-232
  return mul_div255_px(bv, sv >> 24);
}

// The straight-alpha table (internal.nim:68-74), uploaded once per device:
// tbl[a*256 + c] = min(round(c * (255/a)), 255) evaluated in float64.
struct BlendTables {
  const uint8_t* straight;
};

__device__ __forceinline__ uint32_t premul8(uint32_t sv) {  // internal.nim:86-96
  Px s = unpack(sv);
  if (s.a == 255) return sv;
  return pack((s.r * s.a + 127) / 255, (s.g * s.a + 127) / 255, (s.b * s.a + 127) / 255, s.a);
}
// The device table: the straight-alpha table (256 x 256 bytes, row = alpha),
// then 256 floats v / 255.0f (the float division, done once on the host),
// then SoftLight's D(cb) for cb = v / 255.0f (W3C: a cubic for cb <= 0.25,
// else sqrt(cb); the same float operations, done once on the host).
constexpr size_t kTblUnitOff = 65536, kTblSoftOff = 65536 + 1024, kTblBytes = 65536 + 2048;

__device__ __forceinline__ float small_to_f(uint32_t x) {  // exact for x < 2^23
  return __uint_as_float(0x4B000000u | x) - 8388608.0f;
}

__device__ __forceinline__ Px straight8(const uint8_t* tbl, uint32_t v) {
  Px p = unpack(v);
  const uint8_t* row = tbl + p.a * 256;
  return Px{row[p.r], row[p.g], row[p.b], p.a};
}
// round(c * 255) half away from zero, clamped to 0..255 (0 for NaN), without
// the conversion unit: for every float w in (0, 255], round(w) equals
// floor(w + 0.5) with the sum rounded toward zero (checked exhaustively over
// all 1.13e9 such floats), and adding 1.5 * 2^23 rounding down leaves that
// floor in the low mantissa bits.
__device__ __forceinline__ uint32_t unit_to_u8(float c) {
  const float w = c * 255.0f;
  if (!(w > 0.0f)) return 0u;
  const float t = __fadd_rz(fminf(w, 255.0f), 0.5f);
  return __float_as_uint(__fadd_rd(t, 12582912.0f)) - 0x4B400000u;
}

// n / d rounded to nearest from y = RN(1/d), by the correction step of
// Newton-Raphson division (Markstein, IBM J. Res. Dev. 34(1), 1990; Muller et
// al., Handbook of Floating-Point Arithmetic): q0 = RN(n y) may be more than
// one ulp from n / d, so a first correction q1 = RN(q0 + RN(n - q0 d) y)
// brings it within one ulp; then r1 = n - q1 d is exact (one fused
// multiply-add: the remainder of a faithful quotient is representable) and
// RN(q1 + r1 y) is the correctly rounded quotient (Markstein's theorem: y
// correctly rounded, q1 within one ulp).  One reciprocal serves the three
// channels' divisions by the same denominator.  For the finite normal
// operands of the blend formulas; 0 / 0 gives NaN as the IEEE division does.
__device__ __forceinline__ float div_rcp(float n, float d, float y) {
  const float q0 = n * y;
  const float q1 = fmaf(fmaf(-q0, d, n), y, q0);
  const float r1 = fmaf(-q1, d, n);
  return fmaf(r1, y, q1);
}

// chroma float modes (UNPINNED, W3C Compositing Level 1; same operation order
// as the oracle).
struct F3 {
  float r, g, b;
};
__device__ __forceinline__ float lum3(F3 c) { return 0.3f * c.r + 0.59f * c.g + 0.11f * c.b; }
__device__ __forceinline__ F3 clipColor(F3 c) {
  float l = lum3(c);
  float n = fminf(c.r, fminf(c.g, c.b));
  float x = fmaxf(c.r, fmaxf(c.g, c.b));
  if (n < 0.0f) {
    const float d = l - n, y = __frcp_rn(d);
    c.r = l + div_rcp((c.r - l) * l, d, y);
    c.g = l + div_rcp((c.g - l) * l, d, y);
    c.b = l + div_rcp((c.b - l) * l, d, y);
  }
  if (x > 1.0f) {
    const float d = x - l, y = __frcp_rn(d);
    const float k = 1.0f - l;
    c.r = l + div_rcp((c.r - l) * k, d, y);
    c.g = l + div_rcp((c.g - l) * k, d, y);
    c.b = l + div_rcp((c.b - l) * k, d, y);
  }
  return c;
}
__device__ __forceinline__ F3 setLum(F3 c, float l) {
  float d = l - lum3(c);
  return clipColor(F3{c.r + d, c.g + d, c.b + d});
}
__device__ __forceinline__ float sat3(F3 c) {
  return fmaxf(c.r, fmaxf(c.g, c.b)) - fminf(c.r, fminf(c.g, c.b));
}
__device__ __forceinline__ F3 setSat(F3 c, float s) {
  // the first maximum and the first minimum (strict comparisons in r, g, b
  // order), selected without an indexed array so nothing goes to local memory
  int imax = 0, imin = 0;
  float cmax = c.r, cmin = c.r;
  if (c.g > cmax) { imax = 1; cmax = c.g; }
  if (c.b > cmax) { imax = 2; cmax = c.b; }
  if (c.g < cmin) { imin = 1; cmin = c.g; }
  if (c.b < cmin) { imin = 2; cmin = c.b; }
  if (imax == imin) return F3{0.0f, 0.0f, 0.0f};
  const int imid = 3 - imax - imin;
  const float cmid = imid == 0 ? c.r : (imid == 1 ? c.g : c.b);
  float mid = 0.0f, mx = 0.0f;
  if (cmax > cmin) {
    mid = ((cmid - cmin) * s) / (cmax - cmin);
    mx = s;
  }
  return F3{imax == 0 ? mx : (imid == 0 ? mid : 0.0f), imax == 1 ? mx : (imid == 1 ? mid : 0.0f),
            imax == 2 ? mx : (imid == 2 ? mid : 0.0f)};
}
// W3C SoftLight of one channel; dsl[v] = D(v / 255) (the table above), v the
// backdrop's straight 8-bit value
__device__ __forceinline__ float softLight1(float cb, float cs, const float* dsl, uint32_t v) {
  if (cs <= 0.5f) return cb - ((1.0f - 2.0f * cs) * cb) * (1.0f - cb);
  return cb + (2.0f * cs - 1.0f) * (dsl[v] - cb);
}
// One float mode, inlined where the mode is a compile-time constant (draw).
template <int MODE>
__device__ __forceinline__ uint32_t blendFloatT(const uint8_t* tbl, uint32_t bp, uint32_t sp);

static __device__ __noinline__ uint32_t blendFloat(const uint8_t* tbl, uint32_t bp, uint32_t sp, int mode) {
  Px b8 = straight8(tbl, bp), s8 = straight8(tbl, sp);
  const float* u = reinterpret_cast<const float*>(tbl + kTblUnitOff);  // u[v] = v / 255.0f
  const float* dsl = reinterpret_cast<const float*>(tbl + kTblSoftOff);
  F3 cb{u[b8.r], u[b8.g], u[b8.b]};
  F3 cs{u[s8.r], u[s8.g], u[s8.b]};
  float ab = u[b8.a], as = u[s8.a];
  F3 m;
  switch (mode) {
    case kSoftLight:
      m = F3{softLight1(cb.r, cs.r, dsl, b8.r), softLight1(cb.g, cs.g, dsl, b8.g),
             softLight1(cb.b, cs.b, dsl, b8.b)};
      break;
    case kHue: m = setLum(setSat(cs, sat3(cb)), lum3(cb)); break;
    case kSaturation: m = setLum(setSat(cb, sat3(cs)), lum3(cb)); break;
    case kColor: m = setLum(cs, lum3(cb)); break;
    default: m = setLum(cb, lum3(cs)); break;
  }
  float ao = as + ab * (1.0f - as);
  if (!(ao > 0.0f)) return 0u;
  float k = (1.0f - as) * ab;
  float csr = (1.0f - ab) * cs.r + ab * m.r;
  float csg = (1.0f - ab) * cs.g + ab * m.g;
  float csb = (1.0f - ab) * cs.b + ab * m.b;
  const float yo = __frcp_rn(ao);
  float orr = div_rcp(as * csr + k * cb.r, ao, yo);
  float og = div_rcp(as * csg + k * cb.g, ao, yo);
  float ob = div_rcp(as * csb + k * cb.b, ao, yo);
  return premul8(pack(unit_to_u8(orr), unit_to_u8(og), unit_to_u8(ob), unit_to_u8(ao)));
}

template <int MODE>
__device__ __forceinline__ uint32_t blendFloatT(const uint8_t* tbl, uint32_t bp, uint32_t sp) {
  constexpr int mode = MODE;
  Px b8 = straight8(tbl, bp), s8 = straight8(tbl, sp);
  const float* u = reinterpret_cast<const float*>(tbl + kTblUnitOff);  // u[v] = v / 255.0f
  const float* dsl = reinterpret_cast<const float*>(tbl + kTblSoftOff);
  F3 cb{u[b8.r], u[b8.g], u[b8.b]};
  F3 cs{u[s8.r], u[s8.g], u[s8.b]};
  float ab = u[b8.a], as = u[s8.a];
  F3 m;
  switch (mode) {
    case kSoftLight:
      m = F3{softLight1(cb.r, cs.r, dsl, b8.r), softLight1(cb.g, cs.g, dsl, b8.g),
             softLight1(cb.b, cs.b, dsl, b8.b)};
      break;
    case kHue: m = setLum(setSat(cs, sat3(cb)), lum3(cb)); break;
    case kSaturation: m = setLum(setSat(cb, sat3(cs)), lum3(cb)); break;
    case kColor: m = setLum(cs, lum3(cb)); break;
    default: m = setLum(cb, lum3(cs)); break;
  }
  float ao = as + ab * (1.0f - as);
  if (!(ao > 0.0f)) return 0u;
  float k = (1.0f - as) * ab;
  float csr = (1.0f - ab) * cs.r + ab * m.r;
  float csg = (1.0f - ab) * cs.g + ab * m.g;
  float csb = (1.0f - ab) * cs.b + ab * m.b;
  const float yo = __frcp_rn(ao);
  float orr = div_rcp(as * csr + k * cb.r, ao, yo);
  float og = div_rcp(as * csg + k * cb.g, ao, yo);
  float ob = div_rcp(as * csb + k * cb.b, ao, yo);
  return premul8(pack(unit_to_u8(orr), unit_to_u8(og), unit_to_u8(ob), unit_to_u8(ao)));
}


// floor(n / d) for integers held exactly in floats, 0 <= n, n + d < 2^24,
// 1 <= d, n / d < 2^21.  rd is rcp.approx(d) (relative error below 2^-22), so
// n * rd is within n/d * 2^-22 < 0.5 of n / d and its floor -- a round-down
// FMA onto 1.5 * 2^23 -- is off by at most one; one exact remainder test
// (n - q * d, an integer below 2^24 in magnitude) corrects it.
__device__ __forceinline__ float rcp_approx(float d) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
  return r;
}
__device__ __forceinline__ uint32_t fdiv_floor(float n, float d, float rd) {
  const float t = __fmaf_rd(n, rd, 12582912.0f);
  const float q = t - 12582912.0f;
  const float rem = fmaf(-q, d, n);
  uint32_t qi = __float_as_uint(t) - 0x4B400000u;
  qi -= rem < 0.0f ? 1u : 0u;
  qi += rem >= d ? 1u : 0u;
  return qi;
}
// ColorBurn / ColorDodge (blends.nim:111-126, :158-173) with the divisions
// done as above: the same integers as the reference's integer divisions.
template <bool BURN>
__device__ __forceinline__ uint32_t blendBurnDodge(const uint8_t* tbl, uint32_t bv, uint32_t sv) {
  const Px bd = straight8(tbl, bv), sr = straight8(tbl, sv);
  auto mix = [](uint32_t b, uint32_t s) -> uint32_t {
    if (BURN) {
      if (b == 255) return 255u;
      if (s == 0) return 0u;
      const float sf = small_to_f(s);
      const uint32_t v = fdiv_floor(small_to_f(255u * (255u - b)), sf, rcp_approx(sf));
      return 255u - (v < 255u ? v : 255u);
    }
    if (b == 0) return 0u;
    if (s == 255) return 255u;
    const float df = small_to_f(255u - s);
    const uint32_t v = fdiv_floor(small_to_f(255u * b), df, rcp_approx(df));
    return v < 255u ? v : 255u;
  };
  const uint32_t mr = mix(bd.r, sr.r), mg = mix(bd.g, sr.g), mb = mix(bd.b, sr.b);
  // alphaFix (blends.nim:18-39): (t0 src + t1 mixed + t2 backdrop) / a / 255 = ... / (255 a)
  const uint32_t sa = sr.a, ba = bd.a;
  const uint32_t a = sa + ba * (255 - sa) / 255;
  if (a == 0) return 0u;
  const float t0 = small_to_f(sa * (255 - ba)), t1 = small_to_f(sa * ba), t2 = small_to_f((255 - sa) * ba);
  const float d = small_to_f(255u * a), rd = rcp_approx(d);
  const float r = fmaf(t0, small_to_f(sr.r), fmaf(t1, small_to_f(mr), t2 * small_to_f(bd.r)));
  const float g = fmaf(t0, small_to_f(sr.g), fmaf(t1, small_to_f(mg), t2 * small_to_f(bd.g)));
  const float b = fmaf(t0, small_to_f(sr.b), fmaf(t1, small_to_f(mb), t2 * small_to_f(bd.b)));
  return premul8(pack(fdiv_floor(r, d, rd), fdiv_floor(g, d, rd), fdiv_floor(b, d, rd), a));
}

// blender(mode)(backdrop, source)  blends.nim:275-299
__device__ __forceinline__ uint32_t blend_px(int mode, const uint8_t* tbl, uint32_t bv, uint32_t sv) {
  switch (mode) {
    case kNormal: return blendNormal(bv, sv);
    case kMask: return blendMaskPx(bv, sv);
    case kOverwrite: return sv;
    default: break;
  }
  Px b = unpack(bv), s = unpack(sv);
  switch (mode) {
    case kDarken: {  // :72-84
      auto f = [](uint32_t bc, uint32_t ba, uint32_t sc, uint32_t sa) {
        uint32_t x = bc + ((255 - ba) * sc) / 255, y = sc + ((255 - sa) * bc) / 255;
        return (x < y ? x : y) & 255u;
      };
      return pack(f(b.r, b.a, s.r, s.a), f(b.g, b.a, s.g, s.a), f(b.b, b.a, s.b, s.a), blendAlpha(b.a, s.a));
    }
    case kMultiply: {  // :86-100
      auto f = [](uint32_t bc, uint32_t ba, uint32_t sc, uint32_t sa) {
        return (((255 - ba) * sc + (255 - sa) * bc + bc * sc) / 255) & 255u;
      };
      return pack(f(b.r, b.a, s.r, s.a), f(b.g, b.a, s.g, s.a), f(b.b, b.a, s.b, s.a), blendAlpha(b.a, s.a));
    }
    case kLighten: {  // :128-140
      auto f = [](uint32_t bc, uint32_t ba, uint32_t sc, uint32_t sa) {
        uint32_t x = bc + ((255 - ba) * sc) / 255, y = sc + ((255 - sa) * bc) / 255;
        return (x > y ? x : y) & 255u;
      };
      return pack(f(b.r, b.a, s.r, s.a), f(b.g, b.a, s.g, s.a), f(b.b, b.a, s.b, s.a), blendAlpha(b.a, s.a));
    }
    case kScreen:  // :142-146
      return pack(screen1(b.r, s.r), screen1(b.g, s.g), screen1(b.b, s.b), blendAlpha(b.a, s.a));
    case kOverlay:  // :175-179
      return pack(hardLight1(s.r, s.a, b.r, b.a), hardLight1(s.g, s.a, b.g, b.a),
                  hardLight1(s.b, s.a, b.b, b.a), blendAlpha(b.a, s.a));
    case kHardLight:  // :184-188
      return pack(hardLight1(b.r, b.a, s.r, s.a), hardLight1(b.g, b.a, s.g, s.a),
                  hardLight1(b.b, b.a, s.b, s.a), blendAlpha(b.a, s.a));
    case kDifference: {  // :190-204; (bc + sc) wraps as uint8
      auto f = [](uint32_t bc, uint32_t ba, uint32_t sc, uint32_t sa) {
        uint32_t m1 = bc * sa, m2 = sc * ba;
        int mn = (int)((m1 < m2 ? m1 : m2) / 255);
        return (uint32_t)((int)((bc + sc) & 255u) - 2 * mn) & 255u;
      };
      return pack(f(b.r, b.a, s.r, s.a), f(b.g, b.a, s.g, s.a), f(b.b, b.a, s.b, s.a), blendAlpha(b.a, s.a));
    }
    case kExclusion: {  // :206-213
      auto f = [](uint32_t bc, uint32_t sc) {
        int v = (int)(bc + sc) - (int)((2 * bc * sc) / 255);
        return (uint32_t)(v > 0 ? v : 0) & 255u;
      };
      return pack(f(b.r, s.r), f(b.g, s.g), f(b.b, s.b), blendAlpha(b.a, s.a));
    }
    case kColorBurn: return blendBurnDodge<true>(tbl, bv, sv);
    case kColorDodge: return blendBurnDodge<false>(tbl, bv, sv);
    case kSoftLight:
    case kHue:
    case kSaturation:
    case kColor:
    case kLuminosity: return blendFloat(tbl, bv, sv, mode);
    case kSubtractMask: {  // :234-239
      uint32_t a = (b.a * (255 - s.a)) / 255;
      return pack((b.r * a) / 255, (b.g * a) / 255, (b.b * a) / 255, a);
    }
    case kExcludeMask: {  // :241-246
      uint32_t a = (b.a > s.a ? b.a : s.a) - (b.a < s.a ? b.a : s.a);
      return pack((s.r * a) / 255, (s.g * a) / 255, (s.b * a) / 255, a);
    }
  }
  return bv;
}

}  // namespace pxg
