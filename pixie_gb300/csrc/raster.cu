// GPU fill pipeline: pixie's commandsToShapes (cubic/quadratic flattening),
// shapesToSegments, computeBounds/snapToPixels, partitionSegments and the
// fillShapes row loop (src/pixie/paths.nim:654-1912), restated for sm_103a.
//
// k_setup   one CTA per fill job: flatten primitives, emit pixie's segments
//           (quantised, oriented, horizontals dropped) in the reference's
//           order, reduce the bounds, derive the partition geometry, each
//           segment's band range and each band's count and AA flag.
// k_rows    one warp per image row: a ballot scan over the segments collects
//           the row's band entries in segment order (clipped to the band as
//           partitionSegments does), then the reference's per-row decision
//           (the non-AA two-edge fill, the trapezoid fast path, or 5-sample
//           coverage with the nonzero/even-odd walk) and the fused
//           coverage -> paint -> blend write of the row.
// Float math is compiled with -fmad=false: every expression keeps the
// reference's float32 operation order.
#include <cfloat>
#include <climits>

#include "pxg_device.cuh"
#include "raster.cuh"

namespace pxg {

static __device__ constexpr float kEps = (float)(0.0001 * 3.141592653589793);  // paths.nim:44
static constexpr long long kIterCap = 1LL << 24;
static constexpr int kSegTile = 1024;  // segment band ranges staged per pass of the band-list build
static constexpr int kBallotBands = 1024;  // band count up to which the ballot band-list build runs

struct V2 {
  float x, y;
};
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return V2{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) { return V2{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ V2 operator*(V2 a, float s) { return V2{a.x * s, a.y * s}; }
__device__ __forceinline__ V2 operator/(V2 a, float s) { return V2{a.x / s, a.y / s}; }
__device__ __forceinline__ float lengthSq(V2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ float length(V2 v) { return sqrtf(lengthSq(v)); }

// ---------------------------------------------------------------------------
// Flattening  paths.nim:677-762
// ---------------------------------------------------------------------------
__device__ __forceinline__ V2 cubicAt(V2 a, V2 c1, V2 c2, V2 to, float t) {
  float t2 = t * t, t3 = t2 * t;
  return a * (((-t3 + 3 * t2) - 3 * t) + 1) + c1 * ((3 * t3 - 6 * t2) + 3 * t) +
         c2 * (-3 * t3 + 3 * t2) + to * (t3);
}
__device__ __forceinline__ V2 cubicDeriv(V2 a, V2 c1, V2 c2, V2 to, float t) {
  float t2 = t * t;
  return a * ((-3 * t2 + 6 * t) - 3) + c1 * ((9 * t2 - 12 * t) + 3) + c2 * (-9 * t2 + 6 * t) +
         to * (3 * t2);
}
__device__ __forceinline__ V2 quadAt(V2 a, V2 c, V2 to, float t) {
  float t2 = t * t;
  return a * ((t2 - 2 * t) + 1) + c * (-2 * t2 + 2 * t) + to * t2;
}

// The adaptive loops of addCubic/addQuadratic (paths.nim:677-762) with the
// halvings of one search evaluated side by side.  After a segment is
// accepted the loop tries steps s0, s0/2, s0/4, ... until one passes the
// error test (or drops to float32 epsilon, which raises).  Every quantity the
// test at level k reads -- next = f(t + s0/2^k), halfway = f(t + s0/2^(k+1)),
// the tangent at t + s0/2^(k+1) -- depends only on (t, s0, prev): halving a
// normal float is exact, so the sequential loop's recomputed `next = halfway`
// and `t + step/4` equal these values bit for bit.  A group of G lanes tests
// levels base..base+G-1 at once; the first level that accepts (or is at or
// below epsilon) is the one the sequential loop would have stopped at.  With
// G = 1 this is the reference's loop unchanged.  Calls emit(prev, next) for
// every segment addSegment keeps (zero-length ones dropped, :669-675);
// returns a JobStatus.  All G lanes of the group run the loop in lockstep.
__device__ __forceinline__ float pow2neg(int k) {  // 2^-k for 0 <= k < 126
  return __int_as_float((127 - k) << 23);
}
template <class Emit>
__device__ int flatten_curve_group(const Prim& p, float ems, int G, int gl, int leader,
                                   unsigned gmask, Emit&& emit) {
  const bool cubic = p.kind == kPrimCubic;
  const V2 at{p.x[0], p.y[0]}, c1{p.x[1], p.y[1]};
  const V2 c2{p.x[2], p.y[2]}, to{cubic ? p.x[3] : p.x[2], cubic ? p.y[3] : p.y[2]};
  float t = 0, s0 = 1;
  bool halfStepping = false;
  V2 prev = at;
  long long rounds = 0;
  while (true) {
    int kdec = 0;
    V2 nxt{0, 0};
    for (int base = 0;; base += G) {
      if (++rounds > kIterCap) return kErrIterLimit;
      const int k = base + gl;
      const float sk = k < 100 ? s0 * pow2neg(k) : 0.0f;
      const bool invalid = sk <= FLT_EPSILON;
      bool accept = false;
      V2 nx{0, 0};
      if (!invalid) {
        const float sh = sk * 0.5f;
        if (cubic) {
          nx = cubicAt(at, c1, c2, to, t + sk);
          const V2 halfway = cubicAt(at, c1, c2, to, t + sh);
          const V2 midpoint = (prev + nx) / 2;
          const V2 lineTangent = midpoint - prev;
          const V2 curveTangent = cubicDeriv(at, c1, c2, to, t + sh);
          const V2 scaled = (curveTangent / length(curveTangent)) * length(lineTangent);
          const float error = lengthSq(midpoint - halfway);
          const float errorTangent = lengthSq(lineTangent - scaled);
          accept = !(error + errorTangent > ems);
        } else {
          nx = quadAt(at, c1, c2, t + sk);
          const V2 halfway = quadAt(at, c1, c2, t + sh);
          const V2 midpoint = (prev + nx) / 2;
          accept = !(lengthSq(midpoint - halfway) > ems);
        }
      }
      const unsigned dec = (__ballot_sync(gmask, invalid || accept) >> leader) & (G == 32 ? 0xffffffffu : ((1u << G) - 1));
      if (dec) {
        const int src = leader + __ffs(dec) - 1;
        if (__shfl_sync(gmask, (int)invalid, src)) return cubic ? kErrCubic : kErrQuad;
        nxt.x = __shfl_sync(gmask, nx.x, src);
        nxt.y = __shfl_sync(gmask, nx.y, src);
        kdec = base + __ffs(dec) - 1;
        break;
      }
    }
    const float step = s0 * pow2neg(kdec);
    if (prev.x - nxt.x != 0.0f || prev.y - nxt.y != 0.0f) emit(prev, nxt);
    t += step;
    if (t == 1) break;
    prev = nxt;
    if (kdec > 0) halfStepping = true;
    s0 = (!cubic && halfStepping) ? nmin(step, 1 - t) : nmin(step * 2, 1 - t);
  }
  return kOk;
}

// Every group of a warp flattens its curves (primitives gid, gid + NG, ...,
// lines skipped) with the search of flatten_curve_group, but the groups step
// together: one search window per iteration of a warp-wide loop, so the warp
// never serialises its groups' divergent loops.  A group that finishes a
// curve starts its next one in the same loop.  emit(p, prev, next) is called
// by every lane of the group for each segment addSegment keeps.  Returns the
// lane's group's error status for the first failing curve it met (kOk if
// none) and that curve's index in errp.
template <class Emit, class Done>
__device__ int flatten_curves_converged(const Prim* P, int np, float ems, int G, int gid, int NG, int gl, int leader,
                                        int& errp, Emit&& emit, Done&& done, uint8_t* rec = nullptr, int cap = 0,
                                        int* nrec = nullptr) {
  const unsigned gbits = G == 32 ? 0xffffffffu : ((1u << G) - 1);
  auto next_curve = [&](int q) {
    while (q < np && P[q].kind == kPrimLine) q += NG;
    return q;
  };
  int p = next_curve(gid);
  bool cubic = false;
  V2 at{0, 0}, c1{0, 0}, c2{0, 0}, to{0, 0}, prev{0, 0};
  float t = 0, s0 = 1;
  bool halfStepping = false;
  int base = 0;
  long long rounds = 0;
  auto start = [&]() {
    if (p >= np) return;
    const Prim& q = P[p];
    cubic = q.kind == kPrimCubic;
    at = V2{q.x[0], q.y[0]};
    c1 = V2{q.x[1], q.y[1]};
    c2 = V2{q.x[2], q.y[2]};
    to = V2{cubic ? q.x[3] : q.x[2], cubic ? q.y[3] : q.y[2]};
    t = 0;
    s0 = 1;
    prev = at;
    halfStepping = false;
    base = 0;
    rounds = 0;
  };
  start();
  int status = kOk;
  while (true) {
    const bool active = p < np;
    if (!__any_sync(0xffffffffu, active)) break;
    const int k = base + gl;
    const float sk = k < 100 ? s0 * pow2neg(k) : 0.0f;
    const bool invalid = sk <= FLT_EPSILON;
    bool accept = false;
    V2 nx{0, 0};
    if (active && !invalid) {
      const float sh = sk * 0.5f;
      if (cubic) {
        nx = cubicAt(at, c1, c2, to, t + sk);
        const V2 halfway = cubicAt(at, c1, c2, to, t + sh);
        const V2 midpoint = (prev + nx) / 2;
        const V2 lineTangent = midpoint - prev;
        const V2 curveTangent = cubicDeriv(at, c1, c2, to, t + sh);
        const V2 scaled = (curveTangent / length(curveTangent)) * length(lineTangent);
        const float error = lengthSq(midpoint - halfway);
        const float errorTangent = lengthSq(lineTangent - scaled);
        accept = !(error + errorTangent > ems);
      } else {
        nx = quadAt(at, c1, c2, t + sk);
        const V2 halfway = quadAt(at, c1, c2, t + sh);
        const V2 midpoint = (prev + nx) / 2;
        accept = !(lengthSq(midpoint - halfway) > ems);
      }
    }
    const unsigned b = __ballot_sync(0xffffffffu, active && (invalid || accept));
    const unsigned mine = (b >> leader) & gbits;
    const int src = leader + (mine ? __ffs(mine) - 1 : 0);
    const int srcInvalid = __shfl_sync(0xffffffffu, (int)invalid, src);
    const float nxx = __shfl_sync(0xffffffffu, nx.x, src);
    const float nxy = __shfl_sync(0xffffffffu, nx.y, src);
    if (!active) continue;
    if (++rounds > kIterCap) {
      status = kErrIterLimit;
      errp = p;
      p = np;
      continue;
    }
    if (!mine) {
      base += G;
      continue;
    }
    if (srcInvalid) {
      status = cubic ? kErrCubic : kErrQuad;
      errp = p;
      p = np;
      continue;
    }
    const int kdec = base + __ffs(mine) - 1;
    if (rec) {  // record the step's halving level for the replay
      if (*nrec < cap && gl == 0) rec[*nrec] = (uint8_t)kdec;
      ++*nrec;
    }
    const float step = s0 * pow2neg(kdec);
    const V2 nxt{nxx, nxy};
    if (prev.x - nxt.x != 0.0f || prev.y - nxt.y != 0.0f) emit(p, prev, nxt);
    t += step;
    if (t == 1) {
      done(p);
      p = next_curve(p + NG);
      start();
      continue;
    }
    prev = nxt;
    if (kdec > 0) halfStepping = true;
    s0 = (!cubic && halfStepping) ? nmin(step, 1 - t) : nmin(step * 2, 1 - t);
    base = 0;
  }
  return status;
}

// The group's curves again from the halving levels the search recorded: the
// accepted point of a step is cubicAt/quadAt at t + s0 * 2^-level, the same
// expression the search evaluated, so the same segments come out without
// the search.  emit and done as for flatten_curves_converged.
template <class Emit, class Done>
__device__ void replay_curves(const Prim* P, int np, int gid, int NG, const uint8_t* rec, int nrec, Emit&& emit,
                              Done&& done) {
  int n = 0;
  for (int p = gid; p < np; p += NG) {
    const Prim& q = P[p];
    if (q.kind == kPrimLine) continue;
    const bool cubic = q.kind == kPrimCubic;
    const V2 at{q.x[0], q.y[0]}, c1{q.x[1], q.y[1]}, c2{q.x[2], q.y[2]};
    const V2 to{cubic ? q.x[3] : q.x[2], cubic ? q.y[3] : q.y[2]};
    float t = 0, s0 = 1;
    bool halfStepping = false;
    V2 prev = at;
    while (true) {
      if (n >= nrec) return;  // a complete record ends with the last curve's t == 1
      const int kdec = rec[n++];
      const float step = s0 * pow2neg(kdec);
      const V2 nxt = cubic ? cubicAt(at, c1, c2, to, t + step) : quadAt(at, c1, c2, t + step);
      if (prev.x - nxt.x != 0.0f || prev.y - nxt.y != 0.0f) emit(p, prev, nxt);
      t += step;
      if (t == 1) break;
      prev = nxt;
      if (kdec > 0) halfStepping = true;
      s0 = (!cubic && halfStepping) ? nmin(step, 1 - t) : nmin(step * 2, 1 - t);
    }
    done(p);
  }
}

// transform + shapesToSegments for one emitted pair (paths.nim:1059-1096).
// vmath quantize(v, 1/256) = sign(v) * floor(|v| / n) * n.
__device__ __forceinline__ float quantize256(float v) {
  const float n = 1.0f / 256;
  float sgn = v >= 0 ? 1.0f : -1.0f;
  return sgn * (floorf(fabsf(v) / n) * n);
}
__device__ __forceinline__ bool make_seg(const PathJob& J, V2 a, V2 b, float4& s, int& w) {
  if (!J.identity) {
    const float* m = J.mat;
    a = V2{m[0] * a.x + m[3] * a.y + m[6], m[1] * a.x + m[4] * a.y + m[7]};
    b = V2{m[0] * b.x + m[3] * b.y + m[6], m[1] * b.x + m[4] * b.y + m[7]};
  }
  a.y = quantize256(a.y);
  b.y = quantize256(b.y);
  if (a.y == b.y) return false;
  w = 1;
  if (a.y > b.y) {
    V2 t = a;
    a = b;
    b = t;
    w = -1;
  }
  s = make_float4(a.x, a.y, b.x, b.y);
  return true;
}

// ---------------------------------------------------------------------------
// Partitions  paths.nim:1127-1262
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool hasFractional(float v) { return v - truncf(v) != 0; }
__device__ __forceinline__ bool segRequiresAA(float4 s) {  // :1149-1160
  return s.x != s.z || hasFractional(s.x) || hasFractional(s.y) || hasFractional(s.w);
}
// bumpy intersects(Segment, Line): the parametric form of internal.nim:36-48
// without the range check on the line parameter; the point is on the segment.
__device__ __forceinline__ bool intersectSegLine(V2 sa, V2 sb, V2 l0, V2 l1, V2& at) {
  V2 s1 = sb - sa, s2 = l1 - l0;
  float den = (-s2.x * s1.y + s1.x * s2.y);
  float t = (s2.x * (sa.y - l0.y) - s2.y * (sa.x - l0.x)) / den;
  if (t >= 0 && t <= 1) {
    at = sa + s1 * t;
    return true;
  }
  return false;
}
__device__ __forceinline__ bool intersectsInside(V2 aa, V2 ab, V2 ba, V2 bb) {  // internal.nim:36-48
  V2 s1 = ab - aa, s2 = bb - ba;
  float den = (-s2.x * s1.y + s1.x * s2.y);
  float s = (-s1.y * (aa.x - ba.x) + s1.x * (aa.y - ba.y)) / den;
  float t = (s2.x * (aa.y - ba.y) - s2.y * (aa.x - ba.x)) / den;
  return s > 0 && s < 1 && t > 0 && t < 1;
}
__device__ __forceinline__ Entry make_entry(float4 s, int w, float top, float bottom) {
  Entry e;
  e.w = w;
  e.pad = 0;
  e.m = 0;
  e.b = 0;
  float d = s.x - s.z;  // initPartitionEntry :1127-1135
  if (d == 0) {
    e.b = s.x;
  } else {
    e.m = (s.y - s.w) / d;
    e.b = s.y - e.m * s.x;
  }
  V2 a{s.x, s.y}, b{s.z, s.w};
  if (a.y <= top && b.y >= bottom) {  // clip :1236-1248
    V2 at{0, 0};
    intersectSegLine(a, b, V2{0, top}, V2{1000, top}, at);
    a = at;
    intersectSegLine(a, b, V2{0, bottom}, V2{1000, bottom}, at);
    b = at;
  }
  e.ax = a.x;
  e.ay = a.y;
  e.bx = b.x;
  e.by = b.y;
  return e;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024).
__device__ long long block_excl_scan(long long v, long long* s_warp, long long& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    long long t = lane < nw ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) s_warp[lane] = t;
  }
  __syncthreads();
  total = s_warp[nw - 1];
  long long before = warp > 0 ? s_warp[warp - 1] : 0;
  __syncthreads();
  return before + x - v;
}

// ---------------------------------------------------------------------------
// k_setup: flatten -> segments -> bounds -> partitions (one CTA per job)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_setup(PathJob* jobs, Arena A, int maxBands) {
  pdl_trigger();  // the row kernel may be set up while this runs; it waits for the segments
  pdl_wait();
  extern __shared__ int dsm[];
  int* bandc = dsm;             // per band: entry count
  int* bandf = dsm + maxBands;  // per band: flags
  __shared__ long long s_warp[32];
  __shared__ long long s_err;
  __shared__ int s_status;
  __shared__ long long s_segbase, s_bandbase, s_nseg, s_listbase;
  __shared__ uint2 s_tile[kSegTile];
  __shared__ uint32_t s_lohi[66];
  __shared__ float s_red[4][32];
  __shared__ long long s_hdr[6];

  PathJob& J = jobs[blockIdx.x];
  const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const unsigned lt32 = (1u << lane) - 1;
  if (tid == 0) {
    s_err = LLONG_MAX;
    s_status = kOk;
  }
  __syncthreads();

  const Prim* P = J.prims + J.prim_off;
  const int np = J.nprims;
  int* PC = A.primcnt + J.pc_off;
  // curves: groups of G lanes (G divides 32), one curve per group at a time
  const int G = J.group;
  const int NG = T / G, gid = tid / G, gl = tid % G, leader = lane - gl;
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1) << leader);

  // Phase A: count the segments each primitive emits
  for (int p = tid; p < np; p += T) {
    if (P[p].kind != kPrimLine) continue;
    float4 s;
    int w;
    V2 a{P[p].x[0], P[p].y[0]}, b{P[p].x[1], P[p].y[1]};
    PC[p] = ((a.x - b.x != 0.0f || a.y - b.y != 0.0f) && make_seg(J, a, b, s, w)) ? 1 : 0;
  }
  // each group's record of halving levels, for the emitting pass to replay
  constexpr int kStepCap = 512;
  uint8_t* rec = nullptr;
  if (A.fsteps && ((long long)blockIdx.x + 1) * 256 * kStepCap <= A.fsteps_cap)
    rec = A.fsteps + ((long long)blockIdx.x * 256 + gid) * kStepCap;
  int nrec = 0;
  {
    int cnt = 0, errp = 0;
    const int st = flatten_curves_converged(
        P, np, J.ems, G, gid, NG, gl, leader, errp,
        [&](int, V2 a, V2 b) {
          float4 s;
          int w;
          if (make_seg(J, a, b, s, w)) cnt++;
        },
        [&](int p) {
          if (gl == 0) PC[p] = cnt;
          cnt = 0;
        },
        rec, kStepCap, &nrec);
    if (st != kOk && gl == 0)  // the reference raises at the first failing primitive
      atomicMin(&s_err, ((long long)errp << 8) | st);
  }
  __syncthreads();
  if (s_err != LLONG_MAX) {
    if (tid == 0) J.status = (int)(s_err & 255);
    return;
  }
  // exclusive prefix of the counts, in primitive order
  long long total = 0;
  for (int c0 = 0; c0 < np; c0 += T) {
    const int p = c0 + tid;
    long long v = p < np ? PC[p] : 0, tot;
    long long ex = block_excl_scan(v, s_warp, tot);
    if (p < np) PC[p] = (int)(total + ex);
    total += tot;
  }
  if (tid == 0) {
    unsigned long long base = atomicAdd(&A.counters[kCtrSegs], (unsigned long long)total);
    s_segbase = (long long)base;
    s_nseg = total;
    if ((long long)base + total > A.seg_cap || total > INT_MAX) s_status = kErrArenaFull;
  }
  __syncthreads();
  if (s_status != kOk) {
    if (tid == 0) J.status = s_status;
    return;
  }

  // Phase B: emit the segments in order and reduce the bounds (:1098-1117)
  float xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  auto put = [&](long long o, float4 s, int w) {
    A.segs[o] = s;
    A.segw[o] = w;
    xmin = nmin(xmin, nmin(s.x, s.z));
    xmax = nmax(xmax, nmax(s.x, s.z));
    ymin = nmin(ymin, s.y);
    ymax = nmax(ymax, s.w);
  };
  for (int p = tid; p < np; p += T) {
    if (P[p].kind != kPrimLine) continue;
    float4 s;
    int w;
    V2 a{P[p].x[0], P[p].y[0]}, b{P[p].x[1], P[p].y[1]};
    if ((a.x - b.x != 0.0f || a.y - b.y != 0.0f) && make_seg(J, a, b, s, w)) put(s_segbase + PC[p], s, w);
  }
  {
    int cnt = 0, errp = 0;
    auto emitB = [&](int p, V2 a, V2 b) {
      float4 s;
      int w;
      if (make_seg(J, a, b, s, w)) {
        if (gl == 0) put(s_segbase + PC[p] + cnt, s, w);
        cnt++;
      }
    };
    auto doneB = [&](int) { cnt = 0; };
    // replay where every group of the warp kept its whole record, else search again
    if (__all_sync(0xffffffffu, rec != nullptr && nrec <= kStepCap))
      replay_curves(P, np, gid, NG, rec, nrec, emitB, doneB);
    else
      flatten_curves_converged(P, np, J.ems, G, gid, NG, gl, leader, errp, emitB, doneB);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    xmin = nmin(xmin, __shfl_xor_sync(0xffffffffu, xmin, o));
    xmax = nmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
    ymin = nmin(ymin, __shfl_xor_sync(0xffffffffu, ymin, o));
    ymax = nmax(ymax, __shfl_xor_sync(0xffffffffu, ymax, o));
  }
  if (lane == 0) {
    s_red[0][warp] = xmin;
    s_red[1][warp] = xmax;
    s_red[2][warp] = ymin;
    s_red[3][warp] = ymax;
  }
  __syncthreads();

  // Phase C: bounds -> pixel window, partition geometry (:1602-1619, :1172-1192)
  const long long W = J.W, H = J.H;
  if (tid == 0) {
    const int nw = (T + 31) >> 5;
    float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    for (int i = 0; i < nw; i++) {
      x0 = nmin(x0, s_red[0][i]);
      x1 = nmax(x1, s_red[1][i]);
      y0 = nmin(y0, s_red[2][i]);
      y1 = nmax(y1, s_red[3][i]);
    }
    float bx = 0, by = 0, bw = 0, bh = 0;
    if (!(isnan(x0) || isnan(x1) || isnan(y0) || isnan(y1))) {
      bx = x0;
      by = y0;
      bw = x1 - x0;
      bh = y1 - y0;
    }
    float sx = floorf(bx), sw = ceilf(bx + bw) - sx;  // snapToPixels common.nim:92-101
    float sy = floorf(by), sh = ceilf(by + bh) - sy;
    long long startX = max(0LL, nim_int(sx)), startY = max(0LL, nim_int(sy));
    long long pathWidth = startX < W ? min(nim_int(sw), W - startX) : 0LL;
    long long pathHeight = min(H, nim_int(sy + sh));
    int status = kOk;
    if (pathWidth == 0) status = kNothing;
    else if (pathWidth < 0) status = kErrIntOverflow;
    long long height = pathHeight - startY;
    long long nseg = s_nseg;
    uint32_t maxP = (uint32_t)max(1LL, height / 4);
    uint32_t numP = min(maxP, (uint32_t)max(1LL, nseg / 2));
    uint32_t ph = (uint32_t)height / numP;
    if (status == kOk && numP > (uint32_t)maxBands) status = kErrArenaFull;
    s_status = status;
    s_hdr[0] = startX;
    s_hdr[1] = startY;
    s_hdr[2] = pathWidth;
    s_hdr[3] = pathHeight;
    s_hdr[4] = numP;
    s_hdr[5] = ph;
    J.seg_off = s_segbase;
    J.nseg = (int)nseg;
    J.startX = startX;
    J.startY = startY;
    J.pathWidth = pathWidth;
    J.pathHeight = pathHeight;
    J.nb = (int)numP;
    J.ph = ph;
  }
  __syncthreads();
  if (s_status != kOk) {
    if (tid == 0) J.status = s_status;
    return;
  }
  const long long startY = s_hdr[1], pathHeight = s_hdr[3];
  const uint32_t numP = (uint32_t)s_hdr[4], ph = (uint32_t)s_hdr[5];
  const long long height = pathHeight - startY;
  const long long nseg = s_nseg, segbase = s_segbase;
  const float fStartY = (float)(uint32_t)startY;

  auto bandRange = [&](float4 s, uint32_t& a, uint32_t& b) {  // partitionRange :1201-1213
    if (numP == 1) {
      a = b = 0;
      return;
    }
    a = nim_u32(nmax(0.0f, s.y - fStartY)) / ph;
    b = nim_u32(nmax(0.0f, s.w - fStartY)) / ph;
    a = min(a, numP - 1);
    b = min(b, numP - 1);
  };
  (void)height;

  // Phase D: each segment's band range (partitionRange :1201-1213), each
  // band's entry count and anti-aliasing flag (:1215-1234).  With at most
  // kBallotBands bands each warp owns a contiguous run of segments and counts
  // its entries per band (the list build below places them); otherwise
  // shared-memory atomics per band.
  const bool ballot = numP <= (uint32_t)kBallotBands && maxBands <= kBallotBands;
  const int NW = T >> 5;
  int* wc = dsm + 2 * maxBands;  // [warp][band]: entries, then each warp's start
  const long long per = ((nseg + NW - 1) / NW + 31) / 32 * 32;
  const long long ws0 = min(nseg, (long long)warp * per), ws1 = min(nseg, ws0 + per);
  int* mine = wc + warp * (int)numP;
  for (uint32_t k = tid; k < numP; k += T) {
    bandc[k] = 0;
    bandf[k] = 0;
  }
  if (ballot)
    for (int k = tid; k < 2 * NW * (int)numP; k += T) wc[k] = 0;  // counts and band masks
  __syncthreads();
  if (ballot) {
    for (long long i = ws0 + lane; i < ws1; i += 32) {
      const float4 sg = A.segs[segbase + i];
      uint32_t a, b;
      bandRange(sg, a, b);
      A.segband[segbase + i] = make_uint2(a, b);
      const bool aa = segRequiresAA(sg);
      for (uint32_t k = a; k <= b; k++) {
        atomicAdd(&mine[k], 1);
        if (aa) atomicOr(&bandf[k], kBandAA);
      }
    }
    __syncthreads();
    for (uint32_t k = tid; k < numP; k += T) {
      int c = 0;
      for (int w = 0; w < NW; w++) c += wc[w * numP + k];
      bandc[k] = c;
    }
  } else {
    for (long long i = tid; i < nseg; i += T) {
      float4 sg = A.segs[segbase + i];
      uint32_t a, b;
      bandRange(sg, a, b);
      A.segband[segbase + i] = make_uint2(a, b);
      bool aa = segRequiresAA(sg);
      for (uint32_t k = a; k <= b; k++) {
        atomicAdd(&bandc[k], 1);
        if (aa) atomicOr(&bandf[k], kBandAA);
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    unsigned long long base = atomicAdd(&A.counters[kCtrBands], (unsigned long long)numP);
    s_bandbase = (long long)base;
    if ((long long)base + numP > A.band_cap) s_status = kErrArenaFull;
  }
  __syncthreads();
  if (s_status != kOk) {
    if (tid == 0) J.status = s_status;
    return;
  }
  // Phase E: each band's entry list, segment indices ascending -- the order in
  // which partitionSegments appends them (:1215-1234).  Offsets by a scan of
  // the counts; then either each warp writes its run's entries (ballot build)
  // or every thread owns bands and walks the segments in order.
  long long etotal = 0;
  for (uint32_t c0 = 0; c0 < numP; c0 += T) {
    const uint32_t k = c0 + tid;
    long long v = k < numP ? bandc[k] : 0, tot;
    long long ex = block_excl_scan(v, s_warp, tot);
    if (k < numP) {
      Band bd;
      bd.off = etotal + ex;  // relative until the base is known
      bd.count = bandc[k];
      bd.flags = bandf[k];
      A.bands[s_bandbase + k] = bd;
      bandc[k] = (int)(etotal + ex);  // cursor
    }
    etotal += tot;
  }
  if (tid == 0) {
    unsigned long long base = atomicAdd(&A.counters[kCtrBandSegs], (unsigned long long)etotal);
    s_listbase = (long long)base;
    if ((long long)base + etotal > A.bandseg_cap || etotal > INT_MAX) s_status = kErrArenaFull;
  }
  __syncthreads();
  if (s_status != kOk) {
    if (tid == 0) J.status = s_status;
    return;
  }
  int* L = A.bandseg + s_listbase;
  for (uint32_t k = tid; k < numP; k += T) A.bands[s_bandbase + k].off += s_listbase;
  if (ballot) {
    // each warp's start in every band: the band's offset plus the earlier
    // warps' entries; then the warp writes its run's entries: O(entries) work
    for (uint32_t k = tid; k < numP; k += T) {
      int run = bandc[k];
      for (int w = 0; w < NW; w++) {
        const int t = wc[w * numP + k];
        wc[w * numP + k] = run;
        run += t;
      }
    }
    __syncthreads();
    // per batch of 32 segments: every lane marks the bands its segment
    // touches in the warp's band masks; a segment's place in band k is the
    // warp's cursor plus the number of lower lanes in k's mask (the reference's
    // append order); each band's lowest lane then advances the cursor and
    // clears the mask
    uint32_t* bm = reinterpret_cast<uint32_t*>(wc + NW * (int)numP) + warp * (int)numP;
    for (long long c0 = ws0; c0 < ws1; c0 += 32) {
      const long long i = c0 + lane;
      const bool valid = i < ws1;
      uint2 r = make_uint2(1u, 0u);  // empty range
      if (valid) r = A.segband[segbase + i];
      const uint32_t bit = 1u << lane;
      for (uint32_t k = r.x; k <= r.y; k++) atomicOr(&bm[k], bit);
      __syncwarp();
      for (uint32_t k = r.x; k <= r.y; k++) L[mine[k] + __popc(bm[k] & lt32)] = (int)i;
      __syncwarp();
      for (uint32_t k = r.x; k <= r.y; k++) {
        const uint32_t m = bm[k];
        if (!(m & lt32)) mine[k] += __popc(m);
      }
      __syncwarp();
      for (uint32_t k = r.x; k <= r.y; k++)
        if (!(bm[k] & lt32)) bm[k] = 0u;
      __syncwarp();
    }
    if (tid == 0) {
      J.band_off = s_bandbase;
      J.status = kOk;
    }
    return;
  }
  for (long long t0 = 0; t0 < nseg; t0 += kSegTile) {
    const int tl = (int)min((long long)kSegTile, nseg - t0);
    uint32_t lo = UINT_MAX, hi = 0;
    for (int j = tid; j < tl; j += T) {
      uint2 r = A.segband[segbase + t0 + j];
      s_tile[j] = r;
      lo = min(lo, r.x);
      hi = max(hi, r.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) {
      s_lohi[warp] = lo;
      s_lohi[32 + warp] = hi;
    }
    __syncthreads();
    if (tid == 0) {
      for (int i = 1; i < (T + 31) / 32; i++) {
        lo = min(lo, s_lohi[i]);
        hi = max(hi, s_lohi[32 + i]);
      }
      s_lohi[64] = lo;
      s_lohi[65] = hi;
    }
    __syncthreads();
    const uint32_t tlo = s_lohi[64], thi = s_lohi[65];
    for (uint32_t k = tid; k < numP; k += T) {
      if (k < tlo || k > thi) continue;
      int cur = bandc[k];
      for (int j = 0; j < tl; j++) {
        const uint2 r = s_tile[j];
        if (r.x <= k && k <= r.y) L[cur++] = (int)(t0 + j);
      }
      bandc[k] = cur;
    }
    __syncthreads();
  }
  if (tid == 0) {
    J.band_off = s_bandbase;
    J.status = kOk;
  }
}

// ---------------------------------------------------------------------------
// k_rows: the per-row loop of fillShapes (:1631-1908), one warp per row
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool shouldFill(int rule, long long count) {  // :1288-1296
  return rule == 0 ? count != 0 : (count % 2 != 0);
}
// The generic blender, kept out of line: the row code calls it from several
// places, and one copy keeps the kernels small enough for the instruction
// cache.  NormalBlend stays inline at every call site.
static __device__ __noinline__ uint32_t blend_any(int mode, const uint8_t* tbl, uint32_t b, uint32_t s) {
  return blend_px(mode, tbl, b, s);
}
__device__ __forceinline__ uint32_t blend_row(int mode, const uint8_t* tbl, uint32_t b, uint32_t s) {
  return mode == kNormal ? blendNormal(b, s) : blend_any(mode, tbl, b, s);
}
// FILL: a fillHits span (:1540-1591)
__device__ __forceinline__ uint32_t op_fill(int mode, const uint8_t* tbl, uint32_t b, uint32_t c) {
  switch (mode) {
    case kOverwrite: return c;
    case kNormal: return (c >> 24) == 255 ? c : blendNormal(b, c);
    case kMask: return (c >> 24) != 255 ? blendMaskPx(b, c) : b;
    default: return blend_any(mode, tbl, b, c);
  }
}
// COV: fillCoverage with coverage k (:1442-1526)
__device__ __forceinline__ uint32_t op_cov(int mode, const uint8_t* tbl, uint32_t b, uint32_t c, uint32_t k) {
  if (mode == kMask) return k != 255 ? blendMaskPx(b, mul_c(c, k)) : b;
  if (k == 0) return b;
  if (mode == kOverwrite) return mul_c(c, k);
  if (mode == kNormal) return blendNormal(b, mul_c(c, k));
  return blend_any(mode, tbl, b, mul_c(c, k));
}

template <int MAXH, int XT>
struct RowScratch {
  static constexpr int SPCAP = 5 * (MAXH / 2 + 2);
  Entry ent[MAXH];  // the band's entries overlapping the row, in segment order
  int idx[MAXH];
  int a0[MAXH], a1[MAXH], a2[MAXH], a3[MAXH], a4[MAXH], a5[MAXH];
  int2 sp[SPCAP];
  int acc[XT + 1];
  int nsp, flag;
};

// Stable rank of element i among n keys (ties keep the original order).
__device__ __forceinline__ int stable_rank_i(const int* keys, int n, int i) {
  int ki = keys[i], r = 0;
  for (int j = 0; j < n; j++) {
    int kj = keys[j];
    r += (kj < ki) || (kj == ki && j < i);
  }
  return r;
}
__device__ __forceinline__ int stable_rank_f(const float* keys, int n, int i) {
  float ki = keys[i];
  int r = 0;
  for (int j = 0; j < n; j++) {
    float kj = keys[j];
    r += (kj < ki) || (kj == ki && j < i);
  }
  return r;
}

// One row of the destination: premultiplied RGBX (4 bytes per pixel), or an
// 8-bit alpha mask (A8) read as (a, a, a, a) and written as the alpha byte.
// A mask render paints a white opaque colour with NormalBlend onto a
// transparent mask, so every pixel keeps four equal channels and the alpha
// byte holds the whole RGBX value.
template <bool A8>
struct PxRef {
  unsigned char* p;
  __device__ __forceinline__ operator uint32_t() const {
    if (A8) return (uint32_t)*p * 0x01010101u;
    return *reinterpret_cast<const uint32_t*>(p);
  }
  __device__ __forceinline__ const PxRef& operator=(uint32_t v) const {
    if (A8) *p = (unsigned char)(v >> 24);
    else *reinterpret_cast<uint32_t*>(p) = v;
    return *this;
  }
};
// base holds pixel x0 (0 for a whole image row; a row slice staged in shared
// memory starts at its first pixel).
template <bool A8>
struct RowPx {
  unsigned char* base;
  long long x0;
  __device__ __forceinline__ PxRef<A8> operator[](long long x) const {
    return PxRef<A8>{base + (x - x0) * (A8 ? 1 : 4)};
  }
};
template <bool A8>
__device__ __forceinline__ RowPx<A8> row_of(const PathJob& J, long long y) {
  return RowPx<A8>{J.img + y * J.W * (A8 ? 1 : 4), 0};
}

// Linear-index clear of [y*W + a, y*W + b) (clearUnsafe :1433-1440 with
// startY == toY).  Pixels before row y are recorded for the cross-row pass.
template <bool A8>
__device__ void clear_span_linear(const PathJob& J, const Arena& A, int job, RowPx<A8> row,
                                  long long y, long long a, long long b, int lane, long long xa,
                                  long long xb) {
  if (a == J.W) return;
  if (b <= a) return;
  for (long long x = max(max(a, 0LL), xa) + lane; x < min(b, xb); x += 32) row[x] = 0u;
  if (a < 0 && lane == 0 && xa == 0) {
    long long lo = y * J.W + a, hi = y * J.W + min(b, 0LL);
    if (lo < 0) lo = 0;
    if (hi > lo) {
      unsigned long long slot = atomicAdd(&A.counters[kCtrXClears], 1ull);
      if ((long long)slot < A.xclear_cap) {
        A.xclears[3 * slot] = job;
        A.xclears[3 * slot + 1] = lo;
        A.xclears[3 * slot + 2] = hi;
      }
    }
  }
}

// The trapezoid path's pixels for one pair of entries, left (Lm, Lb) and
// right (Rm, Rb), crossing the row at tl0/tl1 and tr0/tr1 (:1752-1835), drawn
// within [xa, xb).
template <bool A8>
__device__ __forceinline__ void apply_trap_pair(RowPx<A8> row, int mode, const uint8_t* tbl, uint32_t rgbx,
                                                long long y, long long W, float Lm, float Lb, float Rm,
                                                float Rb, float tl0, float tl1, float tr0, float tr1,
                                                long long xa, long long xb, int lane, unsigned* cnt = nullptr) {
  const float leftMaxX = nmax(tl0, tl1), rightMinX = nmin(tr0, tr1);
  const long long leftCoverEnd = nim_int(ceilf(leftMaxX));
  const long long rightCoverBegin = nim_int(truncf(rightMinX));
  {  // left sliver (:1752-1788)
    const bool inv = tl0 < tl1;
    const float sliverStart = nmin(tl0, tl1), rectStart = leftMaxX;
    const long long xs = nim_int(sliverStart), xe = nim_int(ceilf(rectStart));
    for (long long x = max(max(xs, 0LL), xa) + lane; x < min(min(xe, W), xb); x += 32) {
      float prevPen = x == xs ? sliverStart : (float)x;
      float pen = (float)(x + 1);
      float rightRectArea = 0;
      if (pen > rectStart) {
        rightRectArea = pen - rectStart;
        pen = rectStart;
      }
      float prevPenY = x == xs ? (inv ? (float)y : (float)(y + 1)) : Lm * (float)x + Lb;
      float penY = Lm * pen + Lb;
      float run = pen - prevPen;
      float tri = 0.5f * run * fabsf(penY - prevPenY);
      float rect = inv ? (prevPenY - (float)y) * run : ((float)(y + 1) - prevPenY) * run;
      float area = tri + rect + rightRectArea;
      row[x] = blend_row(mode, tbl, row[x], mul_f(rgbx, area));
      if (cnt) ++*cnt;
    }
  }
  {  // right sliver (:1790-1828)
    const bool inv = tr0 > tr1;
    const float rectEnd = rightMinX, sliverEnd = nmax(tr0, tr1);
    const long long xs = nim_int(rectEnd), xe = nim_int(ceilf(sliverEnd));
    for (long long x = max(max(xs, 0LL), xa) + lane; x < min(min(xe, W), xb); x += 32) {
      float prevPen = x == xs ? rectEnd : (float)x;
      float pen = (float)(x + 1);
      float ap = fabsf(prevPen);
      float leftRectArea = ap - floorf(ap);  // vmath fractional: fractional part of |v|
      if (pen > sliverEnd) pen = sliverEnd;
      float prevPenY = x == xs ? (inv ? (float)(y + 1) : (float)y) : Rm * (float)x + Rb;
      float penY = Rm * pen + Rb;
      float run = pen - prevPen;
      float tri = 0.5f * run * fabsf(penY - prevPenY);
      float rect = inv ? (penY - (float)y) * run : ((float)(y + 1) - penY) * run;
      float area = leftRectArea + tri + rect;
      row[x] = blend_row(mode, tbl, row[x], mul_f(rgbx, area));
      if (cnt) ++*cnt;
    }
  }
  {  // the fully covered middle (:1830-1835)
    long long fb = max(min(max(leftCoverEnd, 0LL), W), xa), fe = min(min(max(rightCoverBegin, 0LL), W), xb);
    for (long long x = fb + lane; x < fe; x += 32) {
      row[x] = op_fill(mode, tbl, row[x], rgbx);
      if (cnt) ++*cnt;
    }
  }
}

// computeCoverage's accumulation of the sample spans (prevAt, at) in 24.8
// fixed point (:1398-1431) and fillCoverage (:1442-1526) over [cx0, cx1), in
// tiles of XT pixels through the difference array acc (XT + 1 ints).
// computeCoverage's accumulation of the sample spans (prevAt, at) in 24.8
// fixed point (:1398-1431) over the pixels [tx0, tx1) (at most XT): leaves
// acc[i] = coverage of pixel tx0 + i, modulo 256.
template <int XT>
__device__ void cov_tile(const int2* sp, int nsp, int sc, long long tx0, long long tx1, int* acc, int lane) {
  const int L = (int)(tx1 - tx0);
  for (int i = lane; i <= L; i += 32) acc[i] = 0;
  __syncwarp();
  for (int j = lane; j < nsp; j += 32) {
    const int2 spj = sp[j];
    int prevAt = spj.x, at = spj.y;
    long long pi = prevAt / 256, ai = at / 256;
    long long fillStart = pi;
    bool crossed = ai != pi;
    int leftCover = crossed ? (prevAt / 256) * 256 + 256 - prevAt : at - prevAt;
    if (leftCover != 0) {
      fillStart++;
      int v = ((leftCover * sc) / 256) & 255;
      if (pi >= tx0 && pi < tx1) {
        atomicAdd(&acc[pi - tx0], v);
        atomicAdd(&acc[pi - tx0 + 1], -v);
      }
    }
    if (crossed) {
      int rightCover = at - (at / 256) * 256;
      if (rightCover > 0) {
        int v = ((rightCover * sc) / 256) & 255;
        if (ai >= tx0 && ai < tx1) {
          atomicAdd(&acc[ai - tx0], v);
          atomicAdd(&acc[ai - tx0 + 1], -v);
        }
      }
    }
    long long fe = ai;
    long long lo = max(fillStart, tx0), hi = min(fe, tx1);
    if (hi > lo) {
      atomicAdd(&acc[lo - tx0], sc);
      atomicAdd(&acc[hi - tx0], -sc);
    }
  }
  __syncwarp();
  // prefix sum of the difference array, 32 entries per step (lane i holds
  // entry c0 + i: no bank conflicts)
  int carry = 0;
  for (int c0 = 0; c0 < L; c0 += 32) {
    const int i = c0 + lane;
    int v = i < L ? acc[i] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    v += carry;
    if (i < L) acc[i] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
  __syncwarp();
}

// fillCoverage (:1442-1526) of the sample spans over [cx0, cx1), in tiles of
// XT pixels through the difference array acc (XT + 1 ints).
template <bool A8, int XT>
__device__ void apply_cov(RowPx<A8> row, int mode, const uint8_t* tbl, uint32_t rgbx, const int2* sp, int nsp,
                          int sc, long long cx0, long long cx1, int* acc, int lane, unsigned* cnt = nullptr) {
  const bool maskMode = mode == kMask;
  for (long long tx0 = cx0; tx0 < cx1; tx0 += XT) {
    const long long tx1 = min(tx0 + (long long)XT, cx1);
    const int L = (int)(tx1 - tx0);
    cov_tile<XT>(sp, nsp, sc, tx0, tx1, acc, lane);
    // pixels op_cov leaves unchanged are neither read nor written; the next
    // pixel's backdrop is loaded while the current one is blended
    {
      const uint32_t keep = maskMode ? 255u : 0u;
      uint32_t cvN = lane < L ? ((uint32_t)acc[lane] & 255u) : keep;
      uint32_t bdN = cvN != keep ? (uint32_t)row[tx0 + lane] : 0u;
#pragma unroll 1
      for (int i = lane; i < L; i += 32) {
        const uint32_t cv = cvN, bd = bdN;
        const int in = i + 32;
        cvN = in < L ? ((uint32_t)acc[in] & 255u) : keep;
        bdN = cvN != keep ? (uint32_t)row[tx0 + in] : 0u;
        if (cv != keep) {
          row[tx0 + i] = op_cov(mode, tbl, bd, rgbx, cv);
          if (cnt) ++*cnt;
        }
      }
    }
    __syncwarp();
  }
}

// fillHits (:1540-1591) for a non-mask mode: the single sample's spans are
// sorted and disjoint, so a pixel is inside at most one.
template <bool A8>
__device__ void apply_hits(RowPx<A8> row, int mode, const uint8_t* tbl, uint32_t rgbx, const int2* sp, int nsp,
                           long long xa, long long xb, int lane, unsigned* cnt = nullptr) {
  for (long long x = xa + lane; x < xb; x += 32) {
    bool inside = false;
    for (int j = 0; j < nsp && !inside; j++) {
      long long fs = sp[j].x / 256, fe = sp[j].y / 256;
      if (fe - fs > 0 && x >= fs && x < fe) inside = true;
    }
    if (inside) {
      row[x] = op_fill(mode, tbl, row[x], rgbx);
      if (cnt) ++*cnt;
    }
  }
}

// Row programs: what a row of a path draws, recorded by the scene's first
// pass and replayed by its second.  A program is a header unit then data:
//   kRecFill  [minX, maxX) filled            (the non-AA two-edge case)
//   kRecCov   n sample spans, coverage step  (computeCoverage + fillCoverage)
//   kRecHits  n spans                        (fillHits, non-AA)
//   kRecTrap  n pairs: {Lm, Lb, Rm, Rb}, {tl0, tl1, tr0, tr1} per pair
//   kRecCov8  the coverage bytes of pixels [lo, hi), at a 64-bit offset in
//             Arena::cov8 (the accumulation done once, at record time)
enum RecKind { kRecFill = 1, kRecCov = 2, kRecHits = 3, kRecTrap = 4, kRecCov8 = 5 };

// Allocates `units` 16-byte units for row y of job J's program, stores its
// index for the row, and returns it (lane-uniform); -1 if the arena is full.
__device__ __forceinline__ long long rec_alloc(const PathJob& J, const Arena& A, long long y, int units,
                                               int lane) {
  unsigned long long base = 0;
  if (lane == 0) {
    base = atomicAdd(&A.counters[kCtrProg], (unsigned long long)units);
    if ((long long)(base + units) > A.prog_cap || base + units > (unsigned long long)INT_MAX) {
      atomicOr(&A.counters[kCtrProgFull], 1ull);
      A.rowidx[J.ri_off + y * J.ri_stride] = -1;
      base = ~0ull;
    } else {
      A.rowidx[J.ri_off + y * J.ri_stride] = (int)base;
    }
  }
  base = __shfl_sync(0xffffffffu, base, 0);
  return base == ~0ull ? -1 : (long long)base;
}

// Draws the pixels [xa, xb) of row y of job J (the whole row: 0, W).
// Returns false, having drawn nothing, when the row's crossings exceed MAXH
// (the caller retries it with a larger scratch).
// With REC the row is not drawn: its program is recorded instead (non-mask
// modes only).
template <int MAXH, int XT, bool A8, bool REC = false>
__device__ bool process_row(const PathJob& J, const Arena& A, const uint8_t* tbl, int job,
                            long long y, RowScratch<MAXH, XT>& S, int lane, long long xa,
                            long long xb) {
  const long long W = J.W;
  const RowPx<A8> row = row_of<A8>(J, y);
  const int mode = J.mode;
  const uint32_t rgbx = J.rgbx;
  const bool maskMode = mode == kMask;
  const unsigned lt = (1u << lane) - 1;

  long long k = (y - J.startY) / (long long)J.ph;
  if (k >= J.nb) k = J.nb - 1;
  const Band bd = A.bands[J.band_off + k];
  const float scanTop = (float)y, scanBottom = (float)(y + 1);
  // the band's top and bottom (:1178-1190)
  const float top = (float)(J.startY + k * (long long)J.ph);
  const float bottom = (float)(k == J.nb - 1 ? J.pathHeight : J.startY + (k + 1) * (long long)J.ph);
  const float4* SG = A.segs + J.seg_off;
  const int* SW = A.segw + J.seg_off;
  const int* BL = A.bandseg + bd.off;  // the band's segments, ascending
  const int nb = bd.count;
  Entry* E = S.ent;

  // a band of exactly two entries: are they two non-intersecting segments
  // spanning the band (:1250-1262)?
  bool two = false;
  if (nb == 2) {
    if (lane < 2) {
      const int i = BL[lane];
      E[lane] = make_entry(SG[i], SW[i], top, bottom);
    }
    __syncwarp();
    Entry e0 = E[0], e1 = E[1];
    if (!intersectsInside(V2{e0.ax, e0.ay}, V2{e0.bx, e0.by}, V2{e1.ax, e1.ay}, V2{e1.bx, e1.by}) &&
        e0.ay <= top && e0.by >= bottom && e1.ay <= top && e1.by >= bottom) {
      two = true;
      if ((e0.ax + e0.bx) * 0.5f > (e1.ax + e1.bx) * 0.5f) {
        __syncwarp();
        if (lane == 0) {
          E[0] = e1;
          E[1] = e0;
        }
      }
    }
    __syncwarp();
  }

  // (i) non-AA band with two spanning vertical edges (:1644-1668)
  if (two && !(bd.flags & kBandAA)) {
    long long minX = min(max(nim_int(E[0].ax), 0LL), W);
    long long maxX = min(max(nim_int(E[1].ax), 0LL), W);
    if (REC) {
      const long long at = rec_alloc(J, A, y, 1, lane);
      if (at >= 0 && lane == 0) A.prog[at] = make_int4(kRecFill, 0, (int)minX, (int)maxX);
      return true;
    }
    for (long long x = xa + lane; x < xb; x += 32) {
      if (x >= minX && x < maxX) row[x] = op_fill(mode, tbl, row[x], rgbx);
      else if (maskMode) row[x] = 0u;
    }
    return true;
  }

  // entries overlapping the scanline [y, y+1) in band order (:1677-1693)
  int n = 0;
  bool allSpan = true;
  if (two) {
    n = 2;
  } else {
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const int j = c0 + lane;
      bool pred = false, ns = false;
      Entry e;
      if (j < nb) {
        const int i = BL[j];
        e = make_entry(SG[i], SW[i], top, bottom);
        pred = !(e.by <= scanTop || e.ay >= scanBottom);
        ns = e.ay > scanTop || e.by < scanBottom;
      }
      unsigned m = __ballot_sync(0xffffffffu, pred);
      if (__any_sync(0xffffffffu, pred && ns)) allSpan = false;
      int pos = n + __popc(m & lt);
      if (pred && pos < MAXH) E[pos] = e;
      n += __popc(m);
    }
  }
  for (int i = lane; i < min(n, MAXH); i += 32) S.idx[i] = i;
  if (n > MAXH) return false;  // too many crossings for this scratch
  __syncwarp();

  // (ii) trapezoid fast path (:1695-1872)
  if (allSpan && (n % 2) == 0) {
    float* t0 = reinterpret_cast<float*>(S.a0);
    float* t1 = reinterpret_cast<float*>(S.a1);
    float* key = reinterpret_cast<float*>(S.a2);
    bool anyNaN = false;
    for (int i = lane; i < n; i += 32) {
      Entry e = E[S.idx[i]];
      float xt = e.m == 0 ? e.b : (scanTop - e.b) / e.m;   // solveX :1137-1141
      float xbt = e.m == 0 ? e.b : (scanBottom - e.b) / e.m;
      t0[i] = xt;
      t1[i] = xbt;
      key[i] = (xt + xbt) * 0.5f;
      anyNaN |= isnan(key[i]);
    }
    anyNaN = __any_sync(0xffffffffu, anyNaN);
    __syncwarp();
    // stable insertion sort by midpoint (:1710-1719)
    if (anyNaN) {
      if (lane == 0) {
        for (int i = 1; i < n; i++) {
          int j = i - 1, kk = i;
          while (j >= 0 && key[j] > key[kk]) {
            float tk = key[j]; key[j] = key[j + 1]; key[j + 1] = tk;
            float ta = t0[j]; t0[j] = t0[j + 1]; t0[j + 1] = ta;
            float tb = t1[j]; t1[j] = t1[j + 1]; t1[j + 1] = tb;
            int ti = S.idx[j]; S.idx[j] = S.idx[j + 1]; S.idx[j + 1] = ti;
            j--;
            kk--;
          }
        }
      }
    } else {
      float* t0s = reinterpret_cast<float*>(S.a3);
      float* t1s = reinterpret_cast<float*>(S.a4);
      for (int i = lane; i < n; i += 32) {
        int r = stable_rank_f(key, n, i);
        S.a5[r] = S.idx[i];
        t0s[r] = t0[i];
        t1s[r] = t1[i];
      }
      __syncwarp();
      for (int i = lane; i < n; i += 32) {
        S.idx[i] = S.a5[i];
        t0[i] = t0s[i];
        t1[i] = t1s[i];
      }
    }
    __syncwarp();
    // partial coverage of neighbours must not overlap (:1721-1731)
    bool overlap = false;
    for (int i = lane; i < n - 1; i += 32) {
      float leftMaxX = nmax(t0[i], t1[i]);
      float rightMinX = nmin(t0[i + 1], t1[i + 1]);
      if (nim_int(ceilf(leftMaxX)) > nim_int(rightMinX)) overlap = true;
    }
    overlap = __any_sync(0xffffffffu, overlap);
    bool simple = false;
    if (!overlap) {  // pairs must be simple fills (:1733-1750)
      int ok = 1;
      if (lane == 0) {
        long long wc = 0;
        for (int i = 0; i < n; i += 2) {
          wc += E[S.idx[i]].w;
          if (!shouldFill(J.winding, wc)) { ok = 0; break; }
          wc += E[S.idx[i + 1]].w;
          if (shouldFill(J.winding, wc)) { ok = 0; break; }
        }
      }
      simple = __shfl_sync(0xffffffffu, ok, 0) != 0;
    }
    if (simple && REC) {
      const int np = n / 2;
      const long long at = rec_alloc(J, A, y, 1 + 2 * np, lane);
      if (at >= 0) {
        if (lane == 0) A.prog[at] = make_int4(kRecTrap, np, 0, 0);
        for (int p = lane; p < np; p += 32) {
          const Entry L = E[S.idx[2 * p]], R = E[S.idx[2 * p + 1]];
          A.prog[at + 1 + 2 * p] = make_int4(__float_as_int(L.m), __float_as_int(L.b), __float_as_int(R.m),
                                             __float_as_int(R.b));
          A.prog[at + 2 + 2 * p] = make_int4(__float_as_int(t0[2 * p]), __float_as_int(t1[2 * p]),
                                             __float_as_int(t0[2 * p + 1]), __float_as_int(t1[2 * p + 1]));
        }
      }
      return true;
    }
    if (simple) {
      long long filledTo = 0;
      for (int i = 0; i < n; i += 2) {
        const Entry L = E[S.idx[i]], R = E[S.idx[i + 1]];
        const float tl0 = t0[i], tl1 = t1[i], tr0 = t0[i + 1], tr1 = t1[i + 1];
        apply_trap_pair<A8>(row, mode, tbl, rgbx, y, W, L.m, L.b, R.m, R.b, tl0, tl1, tr0, tr1, xa, xb, lane);
        if (maskMode) {  // :1837-1845
          long long clearTo = nim_int(nmin(tl0, tl1));
          clear_span_linear(J, A, job, row, y, min(filledTo, W), min(clearTo, W), lane, xa, xb);
        }
        filledTo = nim_int(ceilf(nmax(tr0, tr1)));
      }
      if (maskMode) clear_span_linear(J, A, job, row, y, min(filledTo, W), W, lane, xa, xb);
      return true;
    }
  }

  // (iii) computeCoverage (:1350-1431) + fillCoverage / fillHits
  const bool aa = (bd.flags & kBandAA) != 0;
  const int quality = aa ? 5 : 1;
  const int sc = 255 / quality;
  const float offset = 1.0f / (float)quality;
  const float initialOffset = offset / 2 + kEps;
  float yLine = (float)y + initialOffset - offset;
  if (lane == 0) S.nsp = 0;
  __syncwarp();
  for (int m = 0; m < quality; m++) {
    yLine += offset;
    int nh = 0;
    for (int c0 = 0; c0 < n; c0 += 32) {
      int i = c0 + lane;
      bool hit = false;
      int fx = 0, w = 0;
      if (i < n) {
        Entry e = E[S.idx[i]];
        if (e.ay <= yLine && e.by >= yLine) {
          hit = true;
          float x = e.m == 0 ? e.b : (yLine - e.b) / e.m;
          fx = nim_i32(nmin(x, (float)W) * 256.0f);
          w = e.w;
        }
      }
      unsigned msk = __ballot_sync(0xffffffffu, hit);
      if (hit) {
        int pos = nh + __popc(msk & lt);
        S.a0[pos] = fx;
        S.a1[pos] = w;
      }
      nh += __popc(msk);
    }
    __syncwarp();
    for (int i = lane; i < nh; i += 32) {  // stable sort (:1277-1286)
      int r = stable_rank_i(S.a0, nh, i);
      S.a2[r] = S.a0[i];
      S.a3[r] = S.a1[i];
    }
    __syncwarp();
    // walk (:1298-1334).  Without two adjacent hits at the same position the
    // look-ahead that skips a cancelling pair never fires, and every hit's
    // part in the walk follows from the winding count before it (a prefix
    // sum): the warp walks 32 hits at a time.  Otherwise lane 0 walks.
    bool adjEq = false;
    for (int i = lane; i + 1 < nh; i += 32) adjEq |= S.a2[i] == S.a2[i + 1];
    if (!__any_sync(0xffffffffu, adjEq)) {
      int ns = S.nsp, carry = 0, prevCarry = 0;
      for (int c0 = 0; c0 < nh; c0 += 32) {
        const int i = c0 + lane;
        const bool valid = i < nh;
        const int at = valid ? S.a2[i] : 0, w = valid ? S.a3[i] : 0;
        int incl = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        const int count = carry + incl - w;
        const bool pos = valid && at > 0;
        const bool fill = shouldFill(J.winding, count);
        const bool shortcut = fill && i < nh - 1 && J.winding == 0 && count + w != 0;
        const bool emit = pos && fill && !shortcut;
        const bool upd = pos && (!fill || emit);  // hits that set prevAt
        const unsigned um = __ballot_sync(0xffffffffu, upd);
        const unsigned below = um & lt;
        const int src = below ? 31 - __clz(below) : lane;
        const int pa = __shfl_sync(0xffffffffu, at, src);
        const int prevAt = below ? pa : prevCarry;
        const unsigned em = __ballot_sync(0xffffffffu, emit);
        const int slot = ns + __popc(em & lt);
        if (emit && slot < RowScratch<MAXH, XT>::SPCAP) S.sp[slot] = make_int2(prevAt, at);
        ns += __popc(em);
        carry += __shfl_sync(0xffffffffu, incl, 31);
        if (um) prevCarry = __shfl_sync(0xffffffffu, at, 31 - __clz(um));
      }
      __syncwarp();
      if (lane == 0) S.nsp = ns;
    } else if (lane == 0) {
      int i = 0, ns = S.nsp;
      long long count = 0;
      int prevAt = 0;
      while (i < nh) {
        int at = S.a2[i], winding = S.a3[i];
        if (at > 0) {
          if (shouldFill(J.winding, count)) {
            if (i < nh - 1) {
              int nextAt = S.a2[i + 1], nextW = S.a3[i + 1];
              if (nextAt == at && winding + nextW == 0) {
                i += 2;
                continue;
              }
              if (J.winding == 0 && count + winding != 0) {
                count += winding;
                i++;
                continue;
              }
            }
            if (ns < RowScratch<MAXH, XT>::SPCAP) S.sp[ns] = make_int2(prevAt, at);
            ns++;
          }
          prevAt = at;
        }
        count += winding;
        i++;
      }
      S.nsp = ns;
    }
    __syncwarp();
  }
  const int nsp = min(S.nsp, RowScratch<MAXH, XT>::SPCAP);

  if (REC) {
    if (nsp > 0 && aa) {
      // the pixels the spans can touch, within the path's bounds
      long long lo = LLONG_MAX, hi = LLONG_MIN;
      for (int j = lane; j < nsp; j += 32) {
        lo = min(lo, (long long)(S.sp[j].x / 256));
        hi = max(hi, (long long)(S.sp[j].y / 256) + 1);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      }
      lo = max(lo, J.startX);
      hi = min(hi, J.startX + J.pathWidth);
      if (hi <= lo) {
        if (lane == 0) A.rowidx[J.ri_off + y * J.ri_stride] = -1;
        return true;
      }
      // coverage bytes when the arena has room (else the spans are recorded)
      const unsigned long long nbytes = (unsigned long long)((hi - lo + 15) & ~15LL);
      unsigned long long cb = 0;
      if (lane == 0) {
        cb = atomicAdd(&A.counters[kCtrCov8], nbytes);
        if ((long long)(cb + nbytes) > A.cov8_cap) cb = ~0ull;
      }
      cb = __shfl_sync(0xffffffffu, cb, 0);
      if (cb != ~0ull) {
        const long long at = rec_alloc(J, A, y, 2, lane);
        if (at < 0) return true;
        if (lane == 0) {
          A.prog[at] = make_int4(kRecCov8, 0, (int)lo, (int)hi);
          A.prog[at + 1] = make_int4((int)(cb & 0xffffffffu), (int)(cb >> 32), 0, 0);
        }
        uint8_t* dst = A.cov8 + cb;
        for (long long tx0 = lo; tx0 < hi; tx0 += XT) {
          const long long tx1 = min(tx0 + (long long)XT, hi);
          cov_tile<XT>(S.sp, nsp, sc, tx0, tx1, S.acc, lane);
          for (int i = lane; i < (int)(tx1 - tx0); i += 32) dst[tx0 - lo + i] = (uint8_t)(S.acc[i] & 255);
          __syncwarp();
        }
        return true;
      }
    }
    const long long at = nsp > 0 ? rec_alloc(J, A, y, 1 + (nsp + 1) / 2, lane) : -1;
    if (nsp == 0 && lane == 0) A.rowidx[J.ri_off + y * J.ri_stride] = -1;
    if (at >= 0) {
      if (lane == 0) A.prog[at] = make_int4(aa ? kRecCov : kRecHits, nsp, sc, 0);
      int2* d = reinterpret_cast<int2*>(A.prog + at + 1);
      for (int j = lane; j < nsp; j += 32) d[j] = S.sp[j];
    }
    return true;
  }
  if (aa) {
    // coverage row over [startX, startX + pathWidth) in tiles of XT pixels
    const long long px0 = J.startX, px1 = J.startX + J.pathWidth;
    if (maskMode) {
      for (long long x = xa + lane; x < xb; x += 32)
        if (x < px0 || x >= px1) row[x] = 0u;
    }
    apply_cov<A8, XT>(row, mode, tbl, rgbx, S.sp, nsp, sc, max(px0, xa), min(px1, xb), S.acc, lane);
  } else if (maskMode) {
    // fillHits with the single sample's spans (:1540-1591); spans are sorted
    // and disjoint, so a pixel is inside at most one.
    const long long startX = J.startX;
    for (long long x = xa + lane; x < xb; x += 32) {
      bool inside = false;
      for (int j = 0; j < nsp && !inside; j++) {
        long long fs = S.sp[j].x / 256, fe = S.sp[j].y / 256;
        if (fe - fs > 0 && x >= fs && x < fe) inside = true;
      }
      row[x] = (x >= startX && inside) ? op_fill(mode, tbl, row[x], rgbx) : 0u;
    }
  } else {
    apply_hits<A8>(row, mode, tbl, rgbx, S.sp, nsp, xa, xb, lane);
  }
  return true;
}

constexpr int kFastMaxH = 256, kFastXT = 1024, kFastWarps = 4;
constexpr int kWideMaxH = 2048, kWideXT = 1024;

// The persistent row kernel: every warp takes work items -- RPI consecutive
// rows of one job -- from a device queue (one atomic per item) until the
// queue is empty, so jobs of uneven height share the GPU evenly.  Rows whose
// crossings exceed MAXH go to the wide kernel.
template <int MAXH, int XT, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_rows(PathJob* jobs, const long long* offs, int njobs, Arena A,
                                                     const uint8_t* tbl, long long totalItems, int rpi) {
  extern __shared__ __align__(16) unsigned char rsm[];
  using Scratch = RowScratch<MAXH, XT>;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Scratch& S = reinterpret_cast<Scratch*>(rsm)[warp];
  pdl_trigger();
  pdl_wait();  // the setup's segments, bands and queue counters
  while (true) {
    unsigned long long q = 0;
    if (lane == 0) q = atomicAdd(&A.counters[kCtrQueue], 1ull);
    const long long item = (long long)__shfl_sync(0xffffffffu, q, 0);
    if (item >= totalItems) break;
    int lo = 0, hi = njobs - 1;  // job with row_off <= item (offs: the jobs' row_off, packed)
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (offs[mid] <= item) lo = mid;
      else hi = mid - 1;
    }
    const PathJob& J = jobs[lo];
    if (J.status != kOk) continue;
    const long long y0 = (item - J.row_off) * rpi;
    for (long long y = y0; y < y0 + rpi && y < J.H; y++) {
      if (y < J.startY || y >= J.pathHeight) {
        if (J.mode == kMask) {  // :1910-1912 (never an A8 job)
          const RowPx<false> row = row_of<false>(J, y);
          for (long long x = lane; x < J.W; x += 32) row[x] = 0u;
        }
        continue;
      }
      const bool ok = J.a8 ? process_row<MAXH, XT, true>(J, A, tbl, lo, y, S, lane, 0, J.W)
                           : process_row<MAXH, XT, false>(J, A, tbl, lo, y, S, lane, 0, J.W);
      if (!ok && lane == 0) {
        // too many crossings for this kernel: hand the row to the wide kernel
        unsigned long long slot = atomicAdd(&A.counters[kCtrOvfRows], 1ull);
        if ((long long)slot < A.ovf_cap) A.ovf_rows[slot] = ((long long)lo << 32) | y;
      }
      __syncwarp();
    }
  }
}

constexpr int kSmallMaxH = 32, kSmallXT = 256, kSmallWarps = 8;
template __global__ void k_rows<kFastMaxH, kFastXT, kFastWarps>(PathJob*, const long long*, int, Arena,
                                                                 const uint8_t*, long long, int);
template __global__ void k_rows<kSmallMaxH, kSmallXT, kSmallWarps>(PathJob*, const long long*, int, Arena,
                                                                   const uint8_t*, long long, int);

// Rows whose crossings exceed the fast kernel's capacity: one warp per CTA
// with room for kWideMaxH crossings.
__global__ void __launch_bounds__(32) k_rows_wide(PathJob* jobs, Arena A, const uint8_t* tbl) {
  extern __shared__ __align__(16) unsigned char rsm[];
  using Scratch = RowScratch<kWideMaxH, kWideXT>;
  Scratch& S = *reinterpret_cast<Scratch*>(rsm);
  const int lane = threadIdx.x & 31;
  long long n = (long long)min((unsigned long long)A.ovf_cap, A.counters[kCtrOvfRows]);
  for (long long i = blockIdx.x; i < n; i += gridDim.x) {
    long long v = A.ovf_rows[i];
    int job = (int)(v >> 32);
    long long y = v & 0xffffffffLL;
    PathJob& J = jobs[job];
    // a row whose band exceeds the wide kernel too reports an error
    long long k = (y - J.startY) / (long long)J.ph;
    if (k >= J.nb) k = J.nb - 1;
    const Band bd = A.bands[J.band_off + k];
    if (bd.count > kWideMaxH) {
      if (lane == 0) J.status = kErrRowTooComplex;
      continue;
    }
    const bool ok = J.a8 ? process_row<kWideMaxH, kWideXT, true>(J, A, tbl, job, y, S, lane, 0, J.W)
                         : process_row<kWideMaxH, kWideXT, false>(J, A, tbl, job, y, S, lane, 0, J.W);
    if (!ok && lane == 0) J.status = kErrRowTooComplex;
  }
}

// Clears that the reference's linear-index clearUnsafe applies to earlier
// rows (a trapezoid fill extending left of the image in MaskBlend); they
// run after every row has been drawn, as they did in the row-ordered loop.
__global__ void k_xclears(PathJob* jobs, Arena A) {
  long long n = (long long)min((unsigned long long)A.xclear_cap, A.counters[kCtrXClears]);
  for (long long i = blockIdx.x; i < n; i += gridDim.x) {
    const PathJob& J = jobs[A.xclears[3 * i]];
    uint32_t* px = reinterpret_cast<uint32_t*>(J.img);
    for (long long p = A.xclears[3 * i + 1] + threadIdx.x; p < A.xclears[3 * i + 2]; p += blockDim.x)
      px[p] = 0u;
  }
}

// Dense scenes, in two passes.
// k_scene_rec: every (path, row) of the launch, independent of the pixels, so
// all of them run in parallel from a device queue: the row's band entries,
// crossings, sort and walk, recorded as the row's program (RecKind).  Rows
// with more crossings than the shared-memory scratch holds take a per-warp
// global-memory scratch of kWideMaxH.
// k_scene: a warp owns a slice of one canvas row (sliceW pixels) and replays
// every path's program for that row in submission order, so each pixel sees
// the paths in the order the reference's sequence of fillPath/strokePath
// calls applies them.  A path that failed in setup stops its run there (the
// reference raises at that call); a path whose bounds miss the slice is
// skipped (outside its bounds a non-mask fill writes nothing).  If the
// program arena overflowed, k_scene draws nothing and the host reruns the
// launch with a larger arena.
constexpr int kRecXT = 256;  // coverage tile of the recording pass
template <int MAXH, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_scene_rec(PathJob* jobs, const SceneRun* runs, int nruns,
                                                          long long totalItems, Arena A, unsigned char* wide,
                                                          long long wideSlots) {
  extern __shared__ __align__(16) unsigned char rsm[];
  using Scratch = RowScratch<MAXH, kRecXT>;
  using Wide = RowScratch<kWideMaxH, kWideXT>;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  pdl_trigger();
  pdl_wait();
  Scratch& S = reinterpret_cast<Scratch*>(rsm)[warp];
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  while (true) {
    unsigned long long q = 0;
    if (lane == 0) q = atomicAdd(&A.counters[kCtrQueue], 1ull);
    const long long item = (long long)__shfl_sync(0xffffffffu, q, 0);
    if (item >= totalItems) break;
    // items run by run, path by path, row by row: rec_off + (j - j0) * H + y
    int r0 = 0, r1 = nruns - 1;
    while (r0 < r1) {
      int mid = (r0 + r1 + 1) >> 1;
      if (runs[mid].rec_off <= item) r0 = mid;
      else r1 = mid - 1;
    }
    const long long local = item - runs[r0].rec_off, H = runs[r0].H;
    const int lo = runs[r0].j0 + (int)(local / H);
    const long long y = local % H;
    const PathJob& J = jobs[lo];
    if (J.status != kOk || y < J.startY || y >= J.pathHeight) continue;
    bool ok = process_row<MAXH, kRecXT, false, true>(J, A, nullptr, lo, y, S, lane, 0, J.W);
    if (!ok && gw < wideSlots) {
      if (lane == 0) atomicAdd(&A.counters[kCtrOvfRows], 1ull);  // rows taking the wide scratch
      __syncwarp();
      ok = process_row<kWideMaxH, kWideXT, false, true>(J, A, nullptr, lo, y, reinterpret_cast<Wide*>(wide)[gw],
                                                        lane, 0, J.W);
    }
    if (!ok && lane == 0) {
      atomicMin(&A.counters[kCtrRowErr], (unsigned long long)lo);
      A.rowidx[J.ri_off + y * J.ri_stride] = -1;
    }
    __syncwarp();
  }
}

template <int XT, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 4) k_scene(PathJob* jobs, const SceneRun* runs, int nruns,
                                                      long long totalItems, Arena A, const uint8_t* tbl,
                                                      int sliceW) {
  __shared__ int accs[WARPS][XT + 1];
  __shared__ uint32_t pix[WARPS][XT];  // the warp's row slice while its paths are applied
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  pdl_trigger();
  pdl_wait();
  int* acc = accs[warp];
  const bool staged = sliceW <= XT;
  if (A.counters[kCtrProgFull]) return;  // programs incomplete: the host reruns the launch
  while (true) {
    unsigned long long q = 0;
    if (lane == 0) q = atomicAdd(&A.counters[kCtrQueue2], 1ull);
    const long long item = (long long)__shfl_sync(0xffffffffu, q, 0);
    if (item >= totalItems) break;
    int lo = 0, hi = nruns - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (runs[mid].row_off <= item) lo = mid;
      else hi = mid - 1;
    }
    const SceneRun R = runs[lo];
    const long long ns = (R.W + sliceW - 1) / sliceW;
    const long long local = item - R.row_off;
    const long long y = local / ns;
    const long long xa = (local % ns) * sliceW, xb = min(xa + sliceW, R.W);
    if (y >= R.H) continue;
    uint32_t* grow = reinterpret_cast<uint32_t*>(R.img) + y * R.W;
    if (staged) {
      for (long long x = xa + lane; x < xb; x += 32) pix[warp][x - xa] = grow[x];
      __syncwarp();
    }
    const RowPx<false> row = staged ? RowPx<false>{reinterpret_cast<unsigned char*>(pix[warp]), xa}
                                    : RowPx<false>{reinterpret_cast<unsigned char*>(grow), 0};
    unsigned painted = 0;  // pixel blends of this item (reported as a launch counter)
    // 32 paths at a time: each lane loads one path's row program index and
    // header (the row's indices are contiguous), then the warp replays the
    // programs in path order.
    const long long rb = R.ri_base + y * (long long)(R.j1 - R.j0);
    for (int c0 = R.j0; c0 < R.j1; c0 += 32) {
      const int j = c0 + lane;
      const bool valid = j < R.j1;
      int st = kNothing, at = -1, mode = 0;
      uint32_t rgbx = 0;
      long long sx = 0, pw = 0;
      if (valid) {
        const PathJob& J = jobs[j];
        st = J.status;
        at = A.rowidx[rb + (j - R.j0)];
        sx = J.startX;
        pw = J.pathWidth;
        mode = J.mode;
        rgbx = J.rgbx;
      }
      // the first failed path stops the run: it and the paths after it draw nothing
      const unsigned bad = __ballot_sync(0xffffffffu, valid && st != kOk && st != kNothing);
      const int lim = bad ? __ffs(bad) - 1 : 32;
      const bool draws = valid && lane < lim && st == kOk && at >= 0 && sx < xb && sx + pw > xa;
      int4 h = make_int4(0, 0, 0, 0);
      if (draws) h = A.prog[at];
      unsigned dm = __ballot_sync(0xffffffffu, draws);
      while (dm) {
        const int i = __ffs(dm) - 1;
        dm &= dm - 1;
        const int hx = __shfl_sync(0xffffffffu, h.x, i), hy = __shfl_sync(0xffffffffu, h.y, i);
        const int hz = __shfl_sync(0xffffffffu, h.z, i), hw = __shfl_sync(0xffffffffu, h.w, i);
        const int ai = __shfl_sync(0xffffffffu, at, i), mi = __shfl_sync(0xffffffffu, mode, i);
        const uint32_t ci = __shfl_sync(0xffffffffu, rgbx, i);
        const long long sxi = __shfl_sync(0xffffffffu, sx, i), pwi = __shfl_sync(0xffffffffu, pw, i);
        if (hx == kRecFill) {
          for (long long x = max((long long)hz, xa) + lane; x < min((long long)hw, xb); x += 32) {
            row[x] = op_fill(mi, tbl, row[x], ci);
            ++painted;
          }
        } else if (hx == kRecCov) {
          apply_cov<false, XT>(row, mi, tbl, ci, reinterpret_cast<const int2*>(A.prog + ai + 1), hy, hz,
                               max(sxi, xa), min(sxi + pwi, xb), acc, lane, &painted);
        } else if (hx == kRecCov8) {
          const int4 u = A.prog[ai + 1];
          const uint8_t* cv8 = A.cov8 + (((long long)(unsigned)u.y << 32) | (unsigned)u.x) - hz;
          const long long x0 = max((long long)hz, xa), x1 = min((long long)hw, xb);
          uint32_t cvN = 0, bdN = 0;
          if (x0 + lane < x1) {
            cvN = cv8[x0 + lane];
            if (cvN) bdN = row[x0 + lane];
          }
#pragma unroll 1
          for (long long x = x0 + lane; x < x1; x += 32) {
            const uint32_t cv = cvN, bd = bdN;
            cvN = 0;
            if (x + 32 < x1) {
              cvN = cv8[x + 32];
              if (cvN) bdN = row[x + 32];
            }
            if (cv) {
              row[x] = op_cov(mi, tbl, bd, ci, cv);
              ++painted;
            }
          }
        } else if (hx == kRecHits) {
          apply_hits<false>(row, mi, tbl, ci, reinterpret_cast<const int2*>(A.prog + ai + 1), hy, xa, xb, lane,
                            &painted);
        } else if (hx == kRecTrap) {
          for (int p = 0; p < hy; p++) {
            const int4 e = A.prog[ai + 1 + 2 * p], t = A.prog[ai + 2 + 2 * p];
            apply_trap_pair<false>(row, mi, tbl, ci, y, R.W, __int_as_float(e.x), __int_as_float(e.y),
                                   __int_as_float(e.z), __int_as_float(e.w), __int_as_float(t.x),
                                   __int_as_float(t.y), __int_as_float(t.z), __int_as_float(t.w), xa, xb, lane,
                                   &painted);
          }
        }
        __syncwarp();
      }
      if (bad) break;
    }
    if (staged) {
      for (long long x = xa + lane; x < xb; x += 32) grow[x] = pix[warp][x - xa];
      __syncwarp();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) painted += __shfl_xor_sync(0xffffffffu, painted, o);
    if (lane == 0 && painted) atomicAdd(&A.counters[kCtrPainted], (unsigned long long)painted);
  }
}

// Scene kernels: the recording pass holds 128 crossings per row in shared
// memory (8 warps per CTA); the drawing pass keeps one 256-pixel coverage
// tile per warp.
constexpr int kRecMaxH = 128, kRecWarps = 8, kSceneXT = 256, kSceneWarps = 8;
const void* scene_rec_kernel() { return (const void*)k_scene_rec<kRecMaxH, kRecWarps>; }
size_t scene_rec_smem() { return sizeof(RowScratch<kRecMaxH, kRecXT>) * kRecWarps; }
int scene_rec_warps() { return kRecWarps; }
const void* scene_kernel() { return (const void*)k_scene<kSceneXT, kSceneWarps>; }
int scene_warps() { return kSceneWarps; }
int scene_tile() { return kSceneXT; }
void launch_scene_rec(unsigned blocks, cudaStream_t st, PathJob* jobs, const SceneRun* runs, int nruns,
                      long long items, const Arena& A, unsigned char* wide, long long slots) {
  launch_pdl(k_scene_rec<kRecMaxH, kRecWarps>, dim3(blocks), dim3(kRecWarps * 32), scene_rec_smem(), st, jobs, runs,
             nruns, items, A, wide, slots);
}
void launch_scene(unsigned blocks, cudaStream_t st, PathJob* jobs, const SceneRun* runs, int nruns, long long items,
                  const Arena& A, const uint8_t* tbl, int sliceW) {
  launch_pdl(k_scene<kSceneXT, kSceneWarps>, dim3(blocks), dim3(kSceneWarps * 32), 0, st, jobs, runs, nruns, items,
             A, tbl, sliceW);
}

// Dynamic shared memory of k_setup for a launch whose images have at most
// maxBands bands: per band a count and flags, plus per warp and band a cursor
// for the ballot band-list build.
size_t setup_smem(int maxBands) {  // counts and flags, then per warp: band counts/cursors and band masks
  return (size_t)maxBands * 8 + (maxBands <= kBallotBands ? (size_t)2 * (256 / 32) * maxBands * 4 : 0);
}

size_t scene_wide_bytes() { return sizeof(RowScratch<kWideMaxH, kWideXT>); }

size_t rows_smem_fast() { return sizeof(RowScratch<kFastMaxH, kFastXT>) * kFastWarps; }
size_t rows_smem_wide() { return sizeof(RowScratch<kWideMaxH, kWideXT>); }
int rows_warps_fast() { return kFastWarps; }

// Row kernel variants: 0 = 256 crossings / 1024-px coverage tiles / 4 warps
// per CTA, 1 = 32 crossings / 256-px tiles / 8 warps (small paths such as
// glyphs: eight times less shared memory per warp, more warps per SM).
const void* rows_kernel(int v) {
  return v == 1 ? (const void*)k_rows<kSmallMaxH, kSmallXT, kSmallWarps>
                : (const void*)k_rows<kFastMaxH, kFastXT, kFastWarps>;
}
size_t rows_smem(int v) {
  return v == 1 ? sizeof(RowScratch<kSmallMaxH, kSmallXT>) * kSmallWarps : rows_smem_fast();
}
int rows_warps(int v) { return v == 1 ? kSmallWarps : kFastWarps; }
void launch_rows(int v, unsigned blocks, cudaStream_t st, PathJob* jobs, const long long* offs, int njobs,
                 const Arena& A, const uint8_t* tbl, long long items, int rpi) {
  if (v == 1)
    launch_pdl(k_rows<kSmallMaxH, kSmallXT, kSmallWarps>, dim3(blocks), dim3(kSmallWarps * 32), rows_smem(1), st, jobs,
               offs, njobs, A, tbl, items, rpi);
  else
    launch_pdl(k_rows<kFastMaxH, kFastXT, kFastWarps>, dim3(blocks), dim3(kFastWarps * 32), rows_smem(0), st, jobs,
               offs, njobs, A, tbl, items, rpi);
}

}  // namespace pxg
