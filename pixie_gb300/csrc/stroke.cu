// Stroke outlines on the GPU: strokeShapes (src/pixie/paths.nim:1922-2082)
// for strokes without dashes.
//
// The host flattens the stroked path into polylines (commandsToShapes, with
// its arcs and the C library's sin/cos) and uploads their points; this kernel
// builds the outline primitives the setup kernel then scan-converts.  One
// thread per polyline point writes that point's fixed slot (raster.cuh,
// StrokeShape): point 0 the start cap, point i >= 1 the rectangle of segment
// i - 1 -> i and the join at i (after the last segment the closing join or
// the end cap).  The slots follow the reference's polygon order, so the
// segments reach the setup kernel in the order the host outline gives them.
//
// Every float32 expression is the host outline's (host_geom.cpp), operation
// for operation (built with -fmad=false; IEEE division and square root).  The
// join's only data-dependent decisions -- skip a straight join, the side of
// the turn, miter or bevel -- compare the turning angle, a difference of two
// atan2f values, with thresholds.  The reference computes it with the C
// library's atan2f; CUDA's atan2f may differ by a few ulps.  A join whose
// angle lies within kAmbiguous of a threshold, where the two could decide
// differently, is written with this kernel's decision and recorded; the host
// recomputes it with the C library and overwrites its slot.  Everywhere else
// both angles fall on the same side of every threshold, so the decisions,
// and the outline, are the reference's.
#include <cstdint>

#include "pxg_device.cuh"
#include "raster.cuh"

namespace pxg {

void note_launch();

namespace {

constexpr double kPI = 3.141592653589793;
constexpr float kEps = (float)(0.0001 * kPI);                       // paths.nim:44
constexpr double kCircleK = 4.0 * (-1.0 + 1.4142135623730951) / 3;  // paths.nim:564
// Bound on |angle (CUDA atan2f) - angle (C library atan2f)|: each atan2f is
// within 3 ulps (CUDA) or 1 ulp (glibc) of the true value, below pi (ulp
// 2.4e-7); the difference and fixAngle's +-2 pi each add half an ulp of 2 pi.
// About 3e-6 in all; 1e-5 leaves a margin of three.
constexpr double kAmbiguous = 1e-5;
enum { kButt = 0, kRoundCap = 1, kSquare = 2 };
enum { kMiter = 0, kRoundJoin = 1, kBevel = 2 };

struct P2 {
  float x, y;
};
__device__ __forceinline__ P2 add(P2 a, P2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ P2 sub(P2 a, P2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ P2 scl(P2 a, float s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ P2 dvd(P2 a, float s) { return {a.x / s, a.y / s}; }
__device__ __forceinline__ float len2(P2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ float len(P2 v) { return sqrtf(len2(v)); }
__device__ __forceinline__ P2 unit(P2 v) { return dvd(v, len(v)); }

__device__ __forceinline__ void put_line(Prim* o, P2 a, P2 b) {
  Prim p;
  p.x[0] = a.x;
  p.y[0] = a.y;
  p.x[1] = b.x;
  p.y[1] = b.y;
  p.x[2] = p.y[2] = p.x[3] = p.y[3] = 0.0f;
  p.kind = kPrimLine;
  p.pad[0] = p.pad[1] = p.pad[2] = 0;
  *o = p;
}
__device__ __forceinline__ void put_pad(Prim* o, int n) {
  for (int k = 0; k < n; k++) put_line(o + k, P2{0.0f, 0.0f}, P2{0.0f, 0.0f});
}
// a closed polygon p[0..n-1], p[n-1] == p[0]: its edges in order (the
// closing pair is the zero-length p[n-1] -> p[0]), padded to 4 primitives
__device__ __forceinline__ void put_poly(Prim* o, const P2* p, int n) {
  int k = 0;
  for (int i = 0; i + 1 < n; i++) put_line(o + k++, p[i], p[i + 1]);
  put_pad(o + k, 4 - k);
}
// makeRect  paths.nim:1943-1965
__device__ __forceinline__ void put_rect(Prim* o, P2 a, P2 b, float hs) {
  const P2 t = unit(sub(b, a));
  const P2 nrm{t.y, t.x};
  const P2 p[5] = {{a.x + nrm.x * hs, a.y - nrm.y * hs}, {b.x + nrm.x * hs, b.y - nrm.y * hs},
                   {b.x - nrm.x * hs, b.y + nrm.y * hs}, {a.x - nrm.x * hs, a.y + nrm.y * hs},
                   {a.x + nrm.x * hs, a.y - nrm.y * hs}};
  put_poly(o, p, 5);
}
// makeCircle  paths.nim:1938-1941: ellipse(c, hs, hs) = Move + 4 cubics + Close,
// which the command walk turns into exactly these four cubic primitives
__device__ __forceinline__ void put_circle(Prim* o, P2 c, float hs) {
  const double mx = kCircleK * (double)hs, my = kCircleK * (double)hs;
  const float cx = c.x, cy = c.y;
  const float q[4][8] = {
      {cx + hs, cy, cx + hs, (float)(cy + my), (float)(cx + mx), cy + hs, cx, cy + hs},
      {cx, cy + hs, (float)(cx - mx), cy + hs, cx - hs, (float)(cy + my), cx - hs, cy},
      {cx - hs, cy, cx - hs, (float)(cy - my), (float)(cx - mx), cy - hs, cx, cy - hs},
      {cx, cy - hs, (float)(cx + mx), cy - hs, cx + hs, (float)(cy - my), cx + hs, cy}};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    Prim p;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      p.x[i] = q[k][2 * i];
      p.y[i] = q[k][2 * i + 1];
    }
    p.kind = kPrimCubic;
    p.pad[0] = p.pad[1] = p.pad[2] = 0;
    o[k] = p;
  }
}
__device__ __forceinline__ float fix_angle(float a) {
  const float tau = (float)(kPI * 2);
  for (int k = 0; k < 4 && (double)a > kPI; k++) a -= tau;
  for (int k = 0; k < 4 && (double)a < -kPI; k++) a += tau;
  return a;
}
// addJoin  paths.nim:1967-2013; returns true when the decision is ambiguous
__device__ bool put_join(Prim* o, P2 prevPos, P2 pos, P2 nextPos, const StrokeShape& S) {
  if (S.join == kRoundJoin) {
    if (S.roundJoin) put_circle(o, pos, S.hs);
    else put_pad(o, 4);
    return false;
  }
  const P2 vn = sub(nextPos, pos), vp = sub(prevPos, pos);
  const float ang = fix_angle(atan2f(vn.y, vn.x) - atan2f(vp.y, vp.x));
  const double d = fabs((double)fabsf(ang) - kPI);
  const bool amb = fabs(d - (double)kEps) < kAmbiguous || fabsf(ang) < (float)kAmbiguous ||
                   (S.join == kMiter && fabs((double)fabsf(ang) - (double)S.miterAngle) < kAmbiguous);
  if (!(d > (double)kEps)) {
    put_pad(o, 4);
    return amb;
  }
  P2 a = scl(unit(sub(pos, prevPos)), S.hs), b = scl(unit(sub(pos, nextPos)), S.hs);
  if (ang >= 0) {
    a = P2{-a.y, a.x};
    b = P2{b.y, -b.x};
  } else {
    a = P2{a.y, -a.x};
    b = P2{-b.y, b.x};
  }
  int lj = S.join;
  if (lj == kMiter && fabsf(ang) < S.miterAngle) lj = kBevel;
  const float minSq = S.minArea * S.minArea;
  if (lj == kMiter) {
    // line(prevPos + a, pos + a) x line(nextPos + b, pos + b)
    const P2 a0 = add(prevPos, a), a1 = add(pos, a), b0 = add(nextPos, b), b1 = add(pos, b);
    const P2 s1 = sub(a1, a0), s2 = sub(b1, b0);
    const float den = (-s2.x * s1.y + s1.x * s2.y);
    if (den != 0) {
      const float t = (s2.x * (a0.y - b0.y) - s2.y * (a0.x - b0.x)) / den;
      const P2 at = add(a0, scl(s1, t));
      const float bls = len2(sub(at, pos));
      const float areaSq = 0.25f * (len2(a) * bls + len2(b) * bls);
      if (areaSq > minSq) {
        const P2 p[5] = {add(pos, a), at, add(pos, b), pos, add(pos, a)};
        put_poly(o, p, 5);
        return amb;
      }
    }
  } else {
    const float areaSq = 0.25f * len2(a) * len2(b);
    if (areaSq > minSq) {
      const P2 p[4] = {add(a, pos), add(b, pos), pos, add(a, pos)};
      put_poly(o, p, 4);
      return amb;
    }
  }
  put_pad(o, 4);
  return amb;
}

// Threads run in blocks of kOutlineThreads consecutive points, and their
// slots are back to back in memory (each shape's slot starts where the one
// before ends), so a block's output is one contiguous range: every thread
// builds its slot in shared memory, then the block writes the range with
// 16-byte stores, consecutive threads on consecutive addresses.
constexpr int kOutlineThreads = 64;
constexpr int kSlotMax = kStrokeSegSlot;  // primitives a thread writes at most
__global__ void __launch_bounds__(kOutlineThreads) k_stroke_outline(const float2* __restrict__ pts,
                                                                    const StrokeShape* __restrict__ shapes,
                                                                    int nshapes, long long nthreads,
                                                                    Prim* __restrict__ out, int2* amb,
                                                                    long long amb_cap,
                                                                    unsigned long long* amb_count) {
  static_assert(sizeof(Prim) == 48, "a primitive is three 16-byte words");
  __shared__ __align__(16) Prim buf[kOutlineThreads * kSlotMax];  // 24 KB
  __shared__ long long s_first[kOutlineThreads + 1];
  for (long long t0 = (long long)blockIdx.x * kOutlineThreads; t0 < nthreads;
       t0 += (long long)gridDim.x * kOutlineThreads) {
    const long long t = t0 + threadIdx.x;
    const bool live = t < nthreads;
    int lo = 0, i = 0;
    long long first = 0;  // this thread's first primitive in `out`
    if (live) {
      int hi = nshapes - 1;  // the last shape whose first thread is <= t
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (shapes[mid].thr_off <= t) lo = mid;
        else hi = mid - 1;
      }
      i = (int)(t - shapes[lo].thr_off);
      first = shapes[lo].prim_off + (i == 0 ? 0 : kStrokeCapSlot + (long long)kStrokeSegSlot * (i - 1));
      s_first[threadIdx.x] = first;
      if (t == nthreads - 1 || threadIdx.x == kOutlineThreads - 1)
        s_first[threadIdx.x + 1] = first + (i == 0 ? kStrokeCapSlot : kStrokeSegSlot);
    }
    __syncthreads();
    const long long base = s_first[0];
    if (live) {
      const StrokeShape S = shapes[lo];
      const int n = S.npts;
      const float2* q = pts + S.pt_off;
      auto P = [&](int k) { return P2{q[k].x, q[k].y}; };
      Prim* o = buf + (first - base);
      if (i == 0) {  // start cap (open polylines)
        if (!S.closed && S.cap == kRoundCap) {
          put_circle(o, P(0), S.hs);
        } else if (!S.closed && S.cap == kSquare) {
          const P2 tg = unit(sub(P(1), P(0)));
          put_rect(o, sub(P(0), scl(tg, S.hs)), P(0), S.hs);
        } else {
          put_pad(o, 4);
        }
      } else {
        put_rect(o, P(i - 1), P(i), S.hs);
        bool ambiguous = false;
        if (i < n - 1) {
          ambiguous = put_join(o + 4, P(i - 1), P(i), P(i + 1), S);
        } else if (S.closed) {
          ambiguous = put_join(o + 4, P(n - 2), P(n - 1), P(1), S);
        } else if (S.cap == kRoundCap) {
          put_circle(o + 4, P(n - 1), S.hs);
        } else if (S.cap == kSquare) {
          const P2 tg = unit(sub(P(n - 1), P(n - 2)));
          put_rect(o + 4, add(P(n - 1), scl(tg, S.hs)), P(n - 1), S.hs);
        } else {
          put_pad(o + 4, 4);
        }
        if (ambiguous) {
          const unsigned long long k = atomicAdd(amb_count, 1ull);
          if ((long long)k < amb_cap) amb[k] = make_int2(lo, i);
        }
      }
    }
    __syncthreads();
    // the block's range [base, end): 16-byte words, consecutive threads on consecutive words
    const long long nlive = nthreads - t0 < kOutlineThreads ? nthreads - t0 : kOutlineThreads;
    const long long words = (s_first[nlive] - base) * 3;
    const uint4* src = reinterpret_cast<const uint4*>(buf);
    uint4* dst = reinterpret_cast<uint4*>(out + base);
    for (long long w = threadIdx.x; w < words; w += kOutlineThreads) dst[w] = src[w];
    __syncthreads();
  }
}

}  // namespace

void launch_stroke_outline(const float2* pts, const StrokeShape* shapes, int nshapes, long long nthreads, Prim* out,
                           int2* amb, long long amb_cap, unsigned long long* amb_count, int nsm, cudaStream_t st) {
  if (nthreads <= 0 || nshapes <= 0) return;
  long long blocks = (nthreads + kOutlineThreads - 1) / kOutlineThreads;
  if (blocks > (long long)nsm * 24) blocks = (long long)nsm * 24;
  k_stroke_outline<<<(unsigned)blocks, kOutlineThreads, 0, st>>>(pts, shapes, nshapes, nthreads, out, amb, amb_cap,
                                                                 amb_count);
  note_launch();
}

}  // namespace pxg
