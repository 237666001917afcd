// draw() with an integer translation (src/pixie/images.nim:468-529 blendRect),
// image fill (images.nim:55-57) and the coverage-free per-pixel blends.
//
// HBM-bound: a draw reads both images and writes the destination (12 B/px;
// Overwrite reads only the source, 8 B/px).  Each thread moves 16-byte
// vectors (4 pixels) when both row layouts allow it; the blend is a
// compile-time template per mode so the inner loop carries no dispatch.
#include <atomic>
#include <initializer_list>
#include <vector>

#include "pxg_device.cuh"
#include "raster.cuh"

namespace pxg {

// Hazards between kernels launched back to back with programmatic dependent
// launch on one stream.  A kernel launched "late" (its `late` argument set)
// does its work without waiting for the kernel before it and executes
// griddepcontrol.wait only before it exits, so its completion still implies
// the completion of every kernel before it; consecutive independent draws and
// blurs then overlap each other's ramp and drain.  A kernel may go late only
// when nothing it writes is read or written, and nothing it reads is written,
// by a kernel that may still be running: every kernel launched since the last
// one that waited at its start (tracked below, per stream).  Any launch that
// does not declare its buffers (note_launch without dep_late) makes the set
// unknown, so the next kernel waits at its start.  The library's callers hold
// its lock, which serialises these calls.
namespace {
struct InFlight {
  cudaStream_t st = nullptr;
  bool unknown = true;
  std::vector<Span> writes, reads;
};
InFlight g_inflight;
bool g_declared = false;  // the next note_launch is the launch dep_late described
bool overlap(const Span& a, const Span& b) {
  const char *pa = static_cast<const char*>(a.p), *pb = static_cast<const char*>(b.p);
  return a.n && b.n && pa < pb + b.n && pb < pa + a.n;
}
bool hits(const Span& x, const std::vector<Span>& set) {
  for (const Span& y : set)
    if (overlap(x, y)) return true;
  return false;
}
}  // namespace

bool dep_late(cudaStream_t st, std::initializer_list<Span> writes, std::initializer_list<Span> reads) {
  InFlight& f = g_inflight;
  bool late = !f.unknown && f.st == st && f.writes.size() + f.reads.size() < 64;
  for (const Span& w : writes) late = late && !hits(w, f.writes) && !hits(w, f.reads);
  for (const Span& r : reads) late = late && !hits(r, f.writes);
  if (!late) {  // this kernel waits at its start: nothing launched before it still runs after that
    f.writes.clear();
    f.reads.clear();
  }
  f.st = st;
  f.unknown = false;
  f.writes.insert(f.writes.end(), writes.begin(), writes.end());
  f.reads.insert(f.reads.end(), reads.begin(), reads.end());
  g_declared = true;
  return late;
}

static std::atomic<unsigned long long> g_launches{0};
void note_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (g_declared)
    g_declared = false;
  else
    g_inflight.unknown = true;
}
unsigned long long launch_count() { return g_launches.load(); }

template <int MODE>
__device__ __forceinline__ uint32_t draw_px(const uint8_t* tbl, uint32_t a, uint32_t b) {
  if (MODE == kNormal) return blendNormal(a, b);
  if (MODE == kOverwrite) return b;
  if (MODE == kMask) return blendMaskPx(a, b);
  if (MODE == kColorBurn) return blendBurnDodge<true>(tbl, a, b);
  if (MODE == kColorDodge) return blendBurnDodge<false>(tbl, a, b);
  if (MODE == kSoftLight || MODE == kHue || MODE == kSaturation || MODE == kColor || MODE == kLuminosity)
    return blendFloatT<MODE>(tbl, a, b);  // the float modes inline, without the mode switch
  return blend_px(MODE, tbl, a, b);
}

// Overlap rectangle: w x h pixels, a at (ax, ay), b at (bx, by).
// vec: rows of both images and both x offsets are multiples of 4 pixels.
template <int MODE>
__global__ void __launch_bounds__(256) k_draw(uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                                              long long Wa, long long Wb, long long ax, long long ay,
                                              long long bx, long long by, long long w, long long h,
                                              const uint8_t* tbl, int vec, int late) {
  pdl_late_entry(late);
  if (vec) {
    // One 16-byte quad (4 pixels) per thread per iteration: the blend is
    // inlined four times, not sixteen, so the float modes keep their code in
    // the instruction cache and their registers low enough for 5-8 resident
    // CTAs, whose warps hide the table gathers and the HBM latency.  The
    // quad's row and column advance by the grid stride without a division.
    const long long qpr = w >> 2;  // quads per row
    const long long nq = qpr * h;
    if (qpr > 0) {
      const long long stride = (long long)gridDim.x * blockDim.x;
      const long long sr = stride / qpr, sc = stride - sr * qpr;
      long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
      long long r = q / qpr, c = q - r * qpr;
      for (; q < nq; q += stride) {
        uint4* pa = reinterpret_cast<uint4*>(a + (ay + r) * Wa + ax + (c << 2));
        const uint4 vb = __ldcs(reinterpret_cast<const uint4*>(b + (by + r) * Wb + bx + (c << 2)));
        uint4 o;
        if (MODE == kOverwrite) {
          o = vb;
        } else {
          const uint4 va = __ldcs(pa);
          o.x = draw_px<MODE>(tbl, va.x, vb.x);
          o.y = draw_px<MODE>(tbl, va.y, vb.y);
          o.z = draw_px<MODE>(tbl, va.z, vb.z);
          o.w = draw_px<MODE>(tbl, va.w, vb.w);
        }
        __stcs(pa, o);
        r += sr;
        c += sc;
        if (c >= qpr) {
          c -= qpr;
          r++;
        }
      }
    }
    // leftover columns (w % 4)
    const long long rem = w & 3;
    if (rem) {
      for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rem * h;
           i += (long long)gridDim.x * blockDim.x) {
        long long r = i / rem, c = (w - rem) + (i - r * rem);
        uint32_t* pa = a + (ay + r) * Wa + ax + c;
        *pa = draw_px<MODE>(tbl, *pa, b[(by + r) * Wb + bx + c]);
      }
    }
  } else {
    const long long n = w * h;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
      long long r = i / w, c = i - r * w;
      uint32_t* pa = a + (ay + r) * Wa + ax + c;
      *pa = draw_px<MODE>(tbl, *pa, b[(by + r) * Wb + bx + c]);
    }
  }
  pdl_late_exit(late);  // completes only after the kernel before it
}

// MaskBlend zeroes the destination outside the overlap (images.nim:473-520):
// the rows above y0 and from y1 down (whole rows, contiguous), then the
// columns left of x0 and from x1 on in rows [y0, y1).  Only those pixels are
// visited.
__global__ void __launch_bounds__(256) k_clear_outside(uint32_t* a, long long Wa, long long Ha,
                                                       long long x0, long long y0, long long x1,
                                                       long long y1, int late) {
  pdl_late_entry(late);
  const long long top = y0 * Wa, bottom = (Ha - y1) * Wa, side = x0 + (Wa - x1), mid = (y1 - y0) * side;
  const long long n = top + bottom + mid;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < top) {
      a[i] = 0u;
    } else if (i < top + bottom) {
      a[y1 * Wa + (i - top)] = 0u;
    } else {
      const long long k = i - top - bottom, r = k / side, c = k - r * side;
      a[(y0 + r) * Wa + (c < x0 ? c : x1 + (c - x0))] = 0u;
    }
  }
  pdl_late_exit(late);
}

// fillUnsafe over the whole image (internal.nim:55-66)
__global__ void __launch_bounds__(256) k_fill(uint32_t* a, long long n, uint32_t c) {
  const long long nq = n >> 2;
  uint4 v = make_uint4(c, c, c, c);
  uint4* a4 = reinterpret_cast<uint4*>(a);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (long long)gridDim.x * blockDim.x)
    a4[i] = v;
  for (long long i = (nq << 2) + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a[i] = c;
}

// blend_px over pixel arrays, for unit-testing the blend modes themselves
__global__ void k_blend_pixels(int mode, const uint8_t* tbl, const uint32_t* bd, const uint32_t* src,
                               uint32_t* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = blend_px(mode, tbl, bd[i], src[i]);
}

typedef void (*DrawKernel)(uint32_t*, const uint32_t*, long long, long long, long long, long long,
                           long long, long long, long long, long long, const uint8_t*, int, int);

template <int M>
struct DrawTable {
  static void fill(DrawKernel* t) {
    t[M] = k_draw<M>;
    DrawTable<M + 1>::fill(t);
  }
};
template <>
struct DrawTable<kNumBlends> {
  static void fill(DrawKernel*) {}
};

DrawKernel draw_kernel(int mode) {
  static DrawKernel table[kNumBlends] = {nullptr};
  if (!table[0]) DrawTable<0>::fill(table);
  return table[mode];
}

// Grid cap of a draw: whole waves of resident CTAs.  The modes with float
// formulas or divisions (ColorBurn, ColorDodge, SoftLight, Hue, Saturation,
// Color, Luminosity) run two waves, the rest one: with consecutive draws
// overlapping (dep_late), a single wave starts every CTA at once and the next
// draw fills the SMs its slowest CTAs leave idle (2048x2048 Normal alone:
// 14.3 us with one wave, 15.3 us with two).
static int draw_grid_cap(int mode, int nsm) {
  static int resident[kNumBlends] = {0};
  if (!resident[mode]) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, draw_kernel(mode), 256, 0) != cudaSuccess || b < 1) b = 1;
    resident[mode] = b;
  }
  const bool heavy = mode == kColorBurn || mode == kColorDodge || mode == kSoftLight || mode == kHue ||
                     mode == kSaturation || mode == kColor || mode == kLuminosity;
  return nsm * resident[mode] * (heavy ? 2 : 1);
}

void launch_draw(uint32_t* a, const uint32_t* b, long long Wa, long long Ha, long long Wb,
                 long long Hb, long long px, long long py, int mode, const uint8_t* tbl, int nsm,
                 cudaStream_t st) {
  // blendRect  images.nim:468-529
  if (px >= Wa || px + Wb <= 0 || py >= Ha || py + Hb <= 0) {
    if (mode == kMask) {
      k_fill<<<nsm * 4, 256, 0, st>>>(a, Wa * Ha, 0u);
      note_launch();
    }
    return;
  }
  long long xStart = px < 0 ? -px : 0, yStart = py < 0 ? -py : 0;
  long long xEnd = Wb < Wa - px ? Wb : Wa - px, yEnd = Hb < Ha - py ? Hb : Ha - py;
  long long w = xEnd - xStart, h = yEnd - yStart;
  long long ax = xStart + px, ay = yStart + py;
  int vec = (Wa % 4 == 0) && (Wb % 4 == 0) && (ax % 4 == 0) && (xStart % 4 == 0);
  long long work = vec ? (w / 4) * h : w * h;
  long long blocks = (work + 255) / 256;
  long long cap = draw_grid_cap(mode, nsm);
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (mode == kMask) {
    const long long outside = Wa * Ha - w * h;  // pixels outside the overlap
    if (outside > 0) {
      long long cb = (outside + 255) / 256;
      if (cb > (long long)nsm * 4) cb = (long long)nsm * 4;
      const int late = dep_late(st, {Span{a, (size_t)(Wa * Ha * 4)}}, {});
      launch_pdl(k_clear_outside, dim3((unsigned)cb), dim3(256), 0, st, a, Wa, Ha, ax, ay, ax + w, ay + h, late);
      note_launch();
    }
  }
  if (w > 0 && h > 0) {
    // the destination is read and written, the source read (the blend tables are constant)
    const int late = dep_late(st, {Span{a, (size_t)(Wa * Ha * 4)}}, {Span{b, (size_t)(Wb * Hb * 4)}});
    launch_pdl(draw_kernel(mode), dim3((unsigned)blocks), dim3(256), 0, st, a, b, Wa, Wb, ax, ay, xStart, yStart, w,
               h, tbl, vec, late);
    note_launch();
  }
}

void launch_fill(uint32_t* a, long long n, uint32_t c, int nsm, cudaStream_t st) {
  long long blocks = (n / 4 + 255) / 256;
  long long cap = (long long)nsm * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_fill<<<(unsigned)blocks, 256, 0, st>>>(a, n, c); note_launch();
}

void launch_blend_pixels(int mode, const uint8_t* tbl, const uint32_t* bd, const uint32_t* src,
                         uint32_t* out, long long n, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  k_blend_pixels<<<(unsigned)blocks, 256, 0, st>>>(mode, tbl, bd, src, out, n); note_launch();
}

// ---------------------------------------------------------------------------
// Ordered composite of a batch of 8-bit masks: for i = 0..n-1,
// draw(page, mask_i as an RGBX image (a, a, a, a), translate(x_i, y_i), mode)
// (images.nim:636-678 with blendRect :468-529).  One CTA owns a TW x TH tile
// of the page; every thread owns TW*TH/256 pixels of it in registers, so the
// masks that overlap the tile are applied to each pixel in batch order with
// no synchronisation between them.  The CTA finds its masks by testing the
// batch's rectangles 256 at a time and compacting the hits in order.
// Tiles no mask touches are neither read nor written.
// ---------------------------------------------------------------------------
template <int TW, int TH>
__global__ void __launch_bounds__(256) k_draw_masks(uint32_t* __restrict__ page, long long W, long long H,
                                                    const MaskDraw* __restrict__ items, int n,
                                                    const uint8_t* __restrict__ masks, int mode,
                                                    const uint8_t* tbl) {
  constexpr int PER = TW * TH / 256;  // pixels per thread
  __shared__ int list[256];
  __shared__ int s_warp[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long tx0 = (long long)blockIdx.x * TW, ty0 = (long long)blockIdx.y * TH;
  const long long tx1 = min(tx0 + TW, W), ty1 = min(ty0 + TH, H);
  uint32_t px[PER];
  bool loaded = false;
  for (int c0 = 0; c0 < n; c0 += 256) {
    const int i = c0 + tid;
    bool hit = false;
    if (i < n) {
      const MaskDraw m = items[i];
      const long long x0 = max(m.x, 0LL), x1 = min(m.x + m.w, W);
      const long long y0 = max(m.y, 0LL), y1 = min(m.y + m.h, H);
      hit = max(x0, tx0) < min(x1, tx1) && max(y0, ty0) < min(y1, ty1);
    }
    const unsigned b = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) s_warp[warp] = __popc(b);
    __syncthreads();
    int before = 0, cnt = 0;
    for (int w = 0; w < 8; w++) {
      if (w < warp) before += s_warp[w];
      cnt += s_warp[w];
    }
    if (hit) list[before + __popc(b & ((1u << lane) - 1))] = i;
    __syncthreads();
    if (cnt > 0) {
      if (!loaded) {
#pragma unroll
        for (int k = 0; k < PER; k++) {
          const int p = tid + 256 * k;
          const long long X = tx0 + p % TW, Y = ty0 + p / TW;
          px[k] = (X < tx1 && Y < ty1) ? page[Y * W + X] : 0u;
        }
        loaded = true;
      }
      for (int j = 0; j < cnt; j++) {
        const MaskDraw m = items[list[j]];
#pragma unroll
        for (int k = 0; k < PER; k++) {
          const int p = tid + 256 * k;
          const long long X = tx0 + p % TW, Y = ty0 + p / TW;
          const long long u = X - m.x, v = Y - m.y;
          if (X < tx1 && Y < ty1 && u >= 0 && u < m.w && v >= 0 && v < m.h) {
            const uint32_t a = (uint32_t)masks[m.off + v * m.w + u] * 0x01010101u;
            px[k] = mode == kNormal ? blendNormal(px[k], a) : (mode == kOverwrite ? a : blend_px(mode, tbl, px[k], a));
          }
        }
      }
    }
    __syncthreads();
  }
  if (loaded) {
#pragma unroll
    for (int k = 0; k < PER; k++) {
      const int p = tid + 256 * k;
      const long long X = tx0 + p % TW, Y = ty0 + p / TW;
      if (X < tx1 && Y < ty1) page[Y * W + X] = px[k];
    }
  }
}

// Tile shapes of the mask composite (the bin size): 0 = 32x32, 1 = 64x32, 2 = 64x64.
int draw_masks_tiles() { return 3; }
void launch_draw_masks(int tile, uint32_t* page, long long W, long long H, const void* items, int n,
                       const uint8_t* masks, int mode, const uint8_t* tbl, cudaStream_t st) {
  const MaskDraw* it = reinterpret_cast<const MaskDraw*>(items);
  if (tile == 0) {
    dim3 grid((unsigned)((W + 31) / 32), (unsigned)((H + 31) / 32));
    k_draw_masks<32, 32><<<grid, 256, 0, st>>>(page, W, H, it, n, masks, mode, tbl);
  } else if (tile == 1) {
    dim3 grid((unsigned)((W + 63) / 64), (unsigned)((H + 31) / 32));
    k_draw_masks<64, 32><<<grid, 256, 0, st>>>(page, W, H, it, n, masks, mode, tbl);
  } else {
    dim3 grid((unsigned)((W + 63) / 64), (unsigned)((H + 63) / 64));
    k_draw_masks<64, 64><<<grid, 256, 0, st>>>(page, W, H, it, n, masks, mode, tbl);
  }
  note_launch();
}
size_t mask_draw_bytes() { return sizeof(MaskDraw); }

}  // namespace pxg
