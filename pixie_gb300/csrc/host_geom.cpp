// Host geometry for the fill/stroke entry points (see host_geom.h).
// Compiled with -ffp-contract=off: float32 expressions keep pixie's operation
// order; a float32 meeting the float64 constant PI is promoted to float64 as
// in Nim, and narrowed where the reference stores it in a float32.
#include "host_geom.h"

#include <cfloat>
#include <cmath>
#include <cstring>

namespace pxg {
namespace {

const double kPI = 3.141592653589793;
const float kEps = (float)(0.0001 * kPI);  // paths.nim:44
const float kMargin = 0.2f;                // paths.nim:45
const double kCircleK = 4.0 * (-1.0 + 1.4142135623730951) / 3;  // paths.nim:564

enum {
  kClose = 0, kMove, kLine, kHLine, kVLine, kCubic, kSCubic, kQuad, kTQuad, kArc,
  kRMove, kRLine, kRHLine, kRVLine, kRCubic, kRSCubic, kRQuad, kRTQuad, kRArc
};
int params_of(int k) {
  static const int pc[19] = {0, 2, 2, 1, 1, 6, 4, 4, 2, 7, 2, 2, 1, 1, 6, 4, 4, 2, 7};
  return pc[k];
}

struct P2 {
  float x, y;
};
inline P2 add(P2 a, P2 b) { return {a.x + b.x, a.y + b.y}; }
inline P2 sub(P2 a, P2 b) { return {a.x - b.x, a.y - b.y}; }
inline P2 scl(P2 a, float s) { return {a.x * s, a.y * s}; }
inline P2 dvd(P2 a, float s) { return {a.x / s, a.y / s}; }
inline bool eq(P2 a, P2 b) { return a.x == b.x && a.y == b.y; }
inline float len2(P2 v) { return v.x * v.x + v.y * v.y; }
inline float len(P2 v) { return sqrtf(len2(v)); }
inline P2 unit(P2 v) { return dvd(v, len(v)); }
inline float fmin_n(float x, float y) { return x <= y ? x : y; }
inline float fmax_n(float x, float y) { return y <= x ? x : y; }

using Poly = std::vector<P2>;

// addSegment  paths.nim:669-675
void seg_into(Poly& poly, P2 a, P2 b) {
  if (a.x - b.x != 0.0f || a.y - b.y != 0.0f) {
    if (poly.empty() || !eq(poly.back(), a)) poly.push_back(a);
    poly.push_back(b);
  }
}

P2 cubic_pt(P2 a, P2 c1, P2 c2, P2 b, float t) {
  float t2 = t * t, t3 = t2 * t;
  P2 r = scl(a, ((-t3 + 3 * t2) - 3 * t) + 1);
  r = add(r, scl(c1, (3 * t3 - 6 * t2) + 3 * t));
  r = add(r, scl(c2, -3 * t3 + 3 * t2));
  return add(r, scl(b, t3));
}
P2 cubic_d(P2 a, P2 c1, P2 c2, P2 b, float t) {
  float t2 = t * t;
  P2 r = scl(a, (-3 * t2 + 6 * t) - 3);
  r = add(r, scl(c1, (9 * t2 - 12 * t) + 3));
  r = add(r, scl(c2, -9 * t2 + 6 * t));
  return add(r, scl(b, 3 * t2));
}
P2 quad_pt(P2 a, P2 c, P2 b, float t) {
  float t2 = t * t;
  return add(add(scl(a, (t2 - 2 * t) + 1), scl(c, -2 * t2 + 2 * t)), scl(b, t2));
}

void flatten_cubic(Poly& poly, P2 a, P2 c1, P2 c2, P2 b, float ems) {  // :677-723
  float t = 0, step = 1;
  P2 prev = a, next = cubic_pt(a, c1, c2, b, t + step), half = cubic_pt(a, c1, c2, b, t + step / 2);
  for (;;) {
    if (step <= FLT_EPSILON) throw GeomError{"Unable to discretize cubic"};
    P2 mid = dvd(add(prev, next), 2);
    P2 lt = sub(mid, prev);
    P2 ct = cubic_d(a, c1, c2, b, t + step / 2);
    P2 cts = scl(unit(ct), len(lt));
    if (len2(sub(mid, half)) + len2(sub(lt, cts)) > ems) {
      next = half;
      half = cubic_pt(a, c1, c2, b, t + step / 4);
      step /= 2;
    } else {
      seg_into(poly, prev, next);
      t += step;
      if (t == 1) break;
      prev = next;
      step = fmin_n(step * 2, 1 - t);
      next = cubic_pt(a, c1, c2, b, t + step);
      half = cubic_pt(a, c1, c2, b, t + step / 2);
    }
  }
}
void flatten_quad(Poly& poly, P2 a, P2 c, P2 b, float ems) {  // :725-762
  float t = 0, step = 1;
  P2 prev = a, next = quad_pt(a, c, b, t + step), half = quad_pt(a, c, b, t + step / 2);
  bool halving = false;
  for (;;) {
    if (step <= FLT_EPSILON) throw GeomError{"Unable to discretize quadratic"};
    P2 mid = dvd(add(prev, next), 2);
    if (len2(sub(mid, half)) > ems) {
      next = half;
      half = quad_pt(a, c, b, t + step / 4);
      halving = true;
      step /= 2;
    } else {
      seg_into(poly, prev, next);
      t += step;
      if (t == 1) break;
      prev = next;
      step = halving ? fmin_n(step, 1 - t) : fmin_n(step * 2, 1 - t);
      next = quad_pt(a, c, b, t + step);
      half = quad_pt(a, c, b, t + step / 2);
    }
  }
}

float svg_angle(P2 u, P2 v) {  // :809-815
  float d = u.x * v.x + u.y * v.y;
  float l = len(u) * len(v);
  float q = d / l;
  float r = acosf(q < -1 ? -1 : (q > 1 ? 1 : q));
  return (u.x * v.y - u.y * v.x) < 0 ? -r : r;
}

void flatten_arc(Poly& poly, P2 at, P2 radiiIn, float rotation, bool large, bool sweep, P2 to,
                 float ems) {  // :764-884
  P2 radii{fabsf(radiiIn.x), fabsf(radiiIn.y)};
  P2 rsq{radii.x * radii.x, radii.y * radii.y};
  const float rad = (float)((double)(rotation / 180.0f) * kPI);
  const float cr = cosf(rad), sr = sinf(rad);
  P2 d{(at.x - to.x) / 2.0f, (at.y - to.y) / 2.0f};
  P2 p{cr * d.x + sr * d.y, -sr * d.x + cr * d.y};
  P2 psq{p.x * p.x, p.y * p.y};
  float c = psq.x / rsq.x + psq.y / rsq.y;
  if (c > 1) {
    radii = scl(radii, sqrtf(c));
    rsq = P2{radii.x * radii.x, radii.y * radii.y};
  }
  float dq = rsq.x * psq.y + rsq.y * psq.x;
  float pq = (rsq.x * rsq.y - dq) / dq;
  float q = sqrtf(fmax_n(0, pq));
  if (large == sweep) q = -q;
  P2 cp{q * radii.x * p.y / radii.y, -q * radii.y * p.x / radii.x};
  P2 center{cr * cp.x - sr * cp.y + (at.x + to.x) / 2, sr * cp.x + cr * cp.y + (at.y + to.y) / 2};
  P2 u{(p.x - cp.x) / radii.x, (p.y - cp.y) / radii.y};
  float theta = svg_angle(P2{1, 0}, u);
  float delta = svg_angle(u, P2{(-p.x - cp.x) / radii.x, (-p.y - cp.y) / radii.y});
  const float tau = (float)(kPI * 2);
  delta = (float)fmod((double)delta, kPI * 2);
  if (sweep && delta < 0) delta += tau;
  else if (!sweep && delta > 0) delta -= tau;
  while ((double)delta > kPI * 2) delta -= tau;
  while ((double)delta < -kPI * 2) delta += tau;
  const float mc = cosf(rad), ms = sinf(rad);
  auto pt = [&](float ang) {  // rotMat * v + center, rotMat = rotate(radians)
    P2 v{cosf(ang) * radii.x, sinf(ang) * radii.y};
    P2 r{mc * v.x + (-ms) * v.y + 0.0f, ms * v.x + mc * v.y + 0.0f};
    return add(r, center);
  };
  float t = 0, step = 1;
  P2 prev = at;
  while (t != 1) {
    if (step <= FLT_EPSILON) throw GeomError{"Unable to discretize arc"};
    float aPrev = theta + delta * t;
    float a = theta + delta * (t + step);
    P2 next = pt(a);
    P2 half = pt(aPrev + (a - aPrev) / 2);
    if (len2(sub(dvd(add(prev, next), 2), half)) > ems) {
      P2 quarter = pt(aPrev + (a - aPrev) / 4);
      if (len2(sub(dvd(add(prev, half), 2), quarter)) < ems) {
        seg_into(poly, prev, half);
        prev = half;
        t += step / 2;
        step = fmin_n(step / 2, 1 - t);
      } else {
        step = step / 4;
      }
    } else {
      seg_into(poly, prev, next);
      prev = next;
      t += step;
      step = fmin_n(step * 2, 1 - t);
    }
  }
}

Prim line_prim(P2 a, P2 b) {
  Prim p;
  memset(&p, 0, sizeof p);
  p.kind = kPrimLine;
  p.x[0] = a.x;
  p.y[0] = a.y;
  p.x[1] = b.x;
  p.y[1] = b.y;
  return p;
}

void emit_polygon_lines(const Poly& poly, std::vector<Prim>& out) {
  // shapesToSegments (:1059-1090): the closing pair (last -> first) comes first.
  if (poly.empty()) return;
  if (!eq(poly.back(), poly.front())) out.push_back(line_prim(poly.back(), poly.front()));
  for (size_t i = 0; i + 1 < poly.size(); i++)
    if (!eq(poly[i], poly[i + 1])) out.push_back(line_prim(poly[i], poly[i + 1]));
}

}  // namespace

void validate_commands(const float* cmds, int64_t n) {
  int64_t i = 0;
  while (i < n) {
    float f = cmds[i];
    if (!(f >= 0 && f <= 18) || f != floorf(f)) throw GeomError{"Invalid path command"};
    int pc = params_of((int)f);
    if (i + 1 + pc > n) throw GeomError{"Invalid path, wrong number of parameters"};
    for (int k = 0; k < pc; k++)
      if (!std::isfinite(cmds[i + 1 + k])) throw GeomError{"Invalid path, non-finite parameter"};
    i += 1 + pc;
  }
}

// commandsToShapes restated (:654-1057).  For strokes (prims == nullptr)
// every subpath is flattened here and returned as a polygon.  For fills the
// subpaths that contain an arc are flattened here and uploaded as lines; the
// others become GPU primitives, with the closing line (Move/Close/end) and,
// for a subpath left open by a relative move, the wrap-around line that
// shapesToSegments adds first (:1072-1080).  An arc-free subpath's polygon
// starts at `start` and ends at `at`, so neither needs host flattening.
static std::vector<Poly> walk_commands(const float* cmd, int64_t n, bool closeSubpaths, float ems,
                                       std::vector<Prim>* prims) {
  const bool gpu = prims != nullptr;
  // subpath regions: a new one begins after Move, RMove and Close
  std::vector<char> regionArc;
  std::vector<int> regionOf;
  if (gpu) {
    int region = 0;
    regionArc.push_back(0);
    for (int64_t i = 0; i < n;) {
      int k = (int)cmd[i];
      if (k == kMove || k == kRMove) {
        regionArc.push_back(0);
        region++;
      }
      regionOf.push_back(region);
      if (k == kArc || k == kRArc) regionArc[(size_t)region] = 1;
      if (k == kClose) {
        regionArc.push_back(0);
        region++;
      }
      i += 1 + params_of(k);
    }
  }
  std::vector<Poly> result;
  P2 start{0, 0}, at{0, 0};
  Poly shape;
  std::vector<Prim> pending;
  bool host = !gpu;  // flatten the current subpath on the host
  int prevKind = kMove;
  P2 prevCtrl{0, 0}, prevCtrl2{0, 0};

  auto finish = [&](bool closing) {
    if (host) {
      if (!shape.empty()) {
        if (closing) seg_into(shape, at, start);
        if (gpu) emit_polygon_lines(shape, *prims);
        else result.push_back(shape);
      }
    } else {
      if (closing) {
        if (!eq(at, start)) pending.push_back(line_prim(at, start));
      } else if (!eq(at, start)) {
        prims->push_back(line_prim(at, start));  // wrap-around pair first
      }
      prims->insert(prims->end(), pending.begin(), pending.end());
    }
    shape.clear();
    pending.clear();
  };
  auto do_line = [&](P2 to) {
    if (host) seg_into(shape, at, to);
    else if (!eq(at, to)) pending.push_back(line_prim(at, to));
  };
  auto do_cubic = [&](P2 c1, P2 c2, P2 to) {
    if (host) {
      flatten_cubic(shape, at, c1, c2, to, ems);
      return;
    }
    Prim p;
    memset(&p, 0, sizeof p);
    p.kind = kPrimCubic;
    p.x[0] = at.x; p.y[0] = at.y; p.x[1] = c1.x; p.y[1] = c1.y;
    p.x[2] = c2.x; p.y[2] = c2.y; p.x[3] = to.x; p.y[3] = to.y;
    pending.push_back(p);
  };
  auto do_quad = [&](P2 c, P2 to) {
    if (host) {
      flatten_quad(shape, at, c, to, ems);
      return;
    }
    Prim p;
    memset(&p, 0, sizeof p);
    p.kind = kPrimQuad;
    p.x[0] = at.x; p.y[0] = at.y; p.x[1] = c.x; p.y[1] = c.y; p.x[2] = to.x; p.y[2] = to.y;
    pending.push_back(p);
  };
  auto do_arc = [&](P2 radii, float rot, bool large, bool sweep, P2 to) {
    flatten_arc(shape, at, radii, rot, large, sweep, to, ems);
  };

  int64_t i = 0;
  size_t ci = 0;
  if (gpu) host = regionArc[0] != 0;
  while (i < n) {
    int kind = (int)cmd[i++];
    const float* c = cmd + i;
    bool cubicPrev = prevKind == kCubic || prevKind == kSCubic || prevKind == kRCubic || prevKind == kRSCubic;
    bool quadPrev = prevKind == kQuad || prevKind == kTQuad || prevKind == kRQuad || prevKind == kRTQuad;
    switch (kind) {
      case kMove:
        finish(closeSubpaths);
        if (gpu) host = regionArc[(size_t)regionOf[ci]] != 0;
        at = P2{c[0], c[1]};
        start = at;
        break;
      case kLine: { P2 to{c[0], c[1]}; do_line(to); at = to; } break;
      case kHLine: { P2 to{c[0], at.y}; do_line(to); at = to; } break;
      case kVLine: { P2 to{at.x, c[0]}; do_line(to); at = to; } break;
      case kCubic: {
        P2 c1{c[0], c[1]}, c2{c[2], c[3]}, to{c[4], c[5]};
        do_cubic(c1, c2, to);
        at = to;
        prevCtrl2 = c2;
      } break;
      case kSCubic: {
        P2 c2{c[0], c[1]}, to{c[2], c[3]};
        P2 c1 = cubicPrev ? sub(scl(at, 2), prevCtrl2) : at;
        do_cubic(c1, c2, to);
        at = to;
        prevCtrl2 = c2;
      } break;
      case kQuad: {
        P2 ct{c[0], c[1]}, to{c[2], c[3]};
        do_quad(ct, to);
        at = to;
        prevCtrl = ct;
      } break;
      case kTQuad: {
        P2 to{c[0], c[1]};
        P2 ct = quadPrev ? sub(scl(at, 2), prevCtrl) : at;
        do_quad(ct, to);
        at = to;
        prevCtrl = ct;
      } break;
      case kArc: {
        P2 to{c[5], c[6]};
        do_arc(P2{c[0], c[1]}, c[2], c[3] == 1, c[4] == 1, to);
        at = to;
      } break;
      case kRMove:
        finish(false);
        if (gpu) host = regionArc[(size_t)regionOf[ci]] != 0;
        at.x += c[0];
        at.y += c[1];
        start = at;
        break;
      case kRLine: { P2 to{at.x + c[0], at.y + c[1]}; do_line(to); at = to; } break;
      case kRHLine: { P2 to{at.x + c[0], at.y}; do_line(to); at = to; } break;
      case kRVLine: { P2 to{at.x, at.y + c[0]}; do_line(to); at = to; } break;
      case kRCubic: {
        P2 c1{at.x + c[0], at.y + c[1]}, c2{at.x + c[2], at.y + c[3]}, to{at.x + c[4], at.y + c[5]};
        do_cubic(c1, c2, to);
        at = to;
        prevCtrl2 = c2;
      } break;
      case kRSCubic: {
        P2 c2{at.x + c[0], at.y + c[1]}, to{at.x + c[2], at.y + c[3]};
        P2 c1 = cubicPrev ? sub(scl(at, 2), prevCtrl2) : at;
        do_cubic(c1, c2, to);
        at = to;
        prevCtrl2 = c2;
      } break;
      case kRQuad: {
        P2 ct{at.x + c[0], at.y + c[1]}, to{at.x + c[2], at.y + c[3]};
        do_quad(ct, to);
        at = to;
        prevCtrl = ct;
      } break;
      case kRTQuad: {
        P2 to{at.x + c[0], at.y + c[1]};
        P2 ct = quadPrev ? sub(scl(at, 2), prevCtrl) : at;
        do_quad(ct, to);
        at = to;
        prevCtrl = ct;
      } break;
      case kRArc: {
        P2 to{at.x + c[5], at.y + c[6]};
        do_arc(P2{c[0], c[1]}, c[2], c[3] == 1, c[4] == 1, to);
        at = to;
      } break;
      case kClose:
        if (!eq(at, start)) {
          do_line(start);
          at = start;
        }
        finish(false);
        if (gpu) host = regionArc[(size_t)regionOf[ci] + 1] != 0;
        break;
    }
    i += params_of(kind);
    prevKind = kind;
    ci++;
  }
  finish(closeSubpaths);
  return result;
}

void build_fill_prims(const float* cmds, int64_t n, float ps, std::vector<Prim>& out) {
  validate_commands(cmds, n);
  out.clear();
  walk_commands(cmds, n, true, error_margin_sq(ps), &out);
}

// ---- strokeShapes  paths.nim:1922-2082 ----------------------------------
namespace {
enum { kButt = 0, kRoundC = 1, kSquare = 2 };
enum { kMiterJ = 0, kRoundJ = 1, kBevelJ = 2 };

struct StrokeCfg {
  float hs, miterAngle, minArea;
  int cap, join;
};
// One outline shape in the reference's order: a polygon of at most 5 points,
// or a circle at c.  Round joins and caps are circles: pixie flattens
// ellipse(c, hs, hs) (:604-616, :1938-1941) with the same error margin, so
// they go to the GPU as their four cubics and are flattened there; the other
// shapes are polygons of lines.
struct OutShape {
  P2 p[5];
  int n;
  bool circ;
  P2 c;
};
OutShape poly_shape(std::initializer_list<P2> pts) {
  OutShape o;
  o.n = 0;
  for (P2 q : pts) o.p[o.n++] = q;
  o.circ = false;
  o.c = P2{0, 0};
  return o;
}
OutShape circle_shape(P2 c) {
  OutShape o;
  o.n = 0;
  o.circ = true;
  o.c = c;
  return o;
}
// The commands of ellipse(c, hs, hs) are Move + 4 cubics + Close, a closed
// arc-free subpath: the command walk turns them into exactly these four cubic
// primitives (the last cubic ends on the start point, so no closing line).
void circle_prims(P2 c, float hs, Prim* out4) {
  const double mx = kCircleK * (double)hs, my = kCircleK * (double)hs;
  const float cx = c.x, cy = c.y;
  const float q[4][8] = {
      {cx + hs, cy, cx + hs, (float)(cy + my), (float)(cx + mx), cy + hs, cx, cy + hs},
      {cx, cy + hs, (float)(cx - mx), cy + hs, cx - hs, (float)(cy + my), cx - hs, cy},
      {cx - hs, cy, cx - hs, (float)(cy - my), (float)(cx - mx), cy - hs, cx, cy - hs},
      {cx, cy - hs, (float)(cx + mx), cy - hs, cx + hs, (float)(cy - my), cx + hs, cy}};
  for (int k = 0; k < 4; k++) {
    Prim p;
    memset(&p, 0, sizeof p);
    p.kind = kPrimCubic;
    for (int i = 0; i < 4; i++) {
      p.x[i] = q[k][2 * i];
      p.y[i] = q[k][2 * i + 1];
    }
    out4[k] = p;
  }
}
OutShape rect_shape(P2 a, P2 b, float hs) {  // :1943-1965
  P2 t = unit(sub(b, a));
  P2 nrm{t.y, t.x};
  P2 p0{a.x + nrm.x * hs, a.y - nrm.y * hs}, p1{b.x + nrm.x * hs, b.y - nrm.y * hs};
  P2 p2{b.x - nrm.x * hs, b.y + nrm.y * hs}, p3{a.x - nrm.x * hs, a.y + nrm.y * hs};
  return poly_shape({p0, p1, p2, p3, p0});
}
float fix_angle(float a) {
  const float tau = (float)(kPI * 2);
  while ((double)a > kPI) a -= tau;
  while ((double)a < -kPI) a += tau;
  return a;
}
// addJoin  :1967-2013; true when a shape was added
bool join_shape(OutShape& o, P2 prevPos, P2 pos, P2 nextPos, const StrokeCfg& c) {
  if (c.join == kRoundJ) {
    float area = (float)kPI * c.hs * c.hs;
    if (area > c.minArea) {
      o = circle_shape(pos);
      return true;
    }
    return false;
  }
  P2 vn = sub(nextPos, pos), vp = sub(prevPos, pos);
  float ang = fix_angle(atan2f(vn.y, vn.x) - atan2f(vp.y, vp.x));
  if (fabs((double)fabsf(ang) - kPI) > (double)kEps) {
    P2 a = scl(unit(sub(pos, prevPos)), c.hs), b = scl(unit(sub(pos, nextPos)), c.hs);
    if (ang >= 0) {
      a = P2{-a.y, a.x};
      b = P2{b.y, -b.x};
    } else {
      a = P2{a.y, -a.x};
      b = P2{-b.y, b.x};
    }
    int lj = c.join;
    if (lj == kMiterJ && fabsf(ang) < c.miterAngle) lj = kBevelJ;
    if (lj == kMiterJ) {
      // line(prevPos + a, pos + a) x line(nextPos + b, pos + b)
      P2 a0 = add(prevPos, a), a1 = add(pos, a), b0 = add(nextPos, b), b1 = add(pos, b);
      P2 s1 = sub(a1, a0), s2 = sub(b1, b0);
      float den = (-s2.x * s1.y + s1.x * s2.y);
      if (den != 0) {
        float t = (s2.x * (a0.y - b0.y) - s2.y * (a0.x - b0.x)) / den;
        P2 at = add(a0, scl(s1, t));
        float bls = len2(sub(at, pos));
        float areaSq = 0.25f * (len2(a) * bls + len2(b) * bls);
        if (areaSq > (c.minArea * c.minArea)) {
          o = poly_shape({add(pos, a), at, add(pos, b), pos, add(pos, a)});
          return true;
        }
      }
    } else if (lj == kBevelJ) {
      float areaSq = 0.25f * len2(a) * len2(b);
      if (areaSq > (c.minArea * c.minArea)) {
        o = poly_shape({add(a, pos), add(b, pos), pos, add(a, pos)});
        return true;
      }
    }
  }
  return false;
}
StrokeCfg stroke_cfg(float ps, float strokeWidth, int lineCap, int lineJoin, float miterLimit) {
  StrokeCfg c;
  c.hs = strokeWidth / 2;
  c.miterAngle = asinf(1 / miterLimit) * 2;
  c.minArea = kMargin / ps;
  c.cap = lineCap;
  c.join = lineJoin;
  return c;
}
}  // namespace

void build_stroke_prims(const float* cmds, int64_t n, float ps, float strokeWidth, int lineCap,
                        int lineJoin, float miterLimit, const float* dashesIn, int64_t nd,
                        std::vector<Prim>& out) {
  validate_commands(cmds, n);
  out.clear();
  const float ems = error_margin_sq(ps);
  std::vector<Poly> shapes = walk_commands(cmds, n, false, ems, nullptr);
  if (strokeWidth <= 0) return;
  const StrokeCfg cfg = stroke_cfg(ps, strokeWidth, lineCap, lineJoin, miterLimit);
  const float hs = cfg.hs;
  auto join = [&](std::vector<OutShape>& o, P2 prevPos, P2 pos, P2 nextPos) {
    OutShape sh;
    if (join_shape(sh, prevPos, pos, nextPos, cfg)) o.push_back(sh);
  };
  std::vector<float> dashes(dashesIn, dashesIn + nd);
  if (dashes.size() % 2 != 0) {
    std::vector<float> d2 = dashes;
    dashes.insert(dashes.end(), d2.begin(), d2.end());
  }
  std::vector<OutShape> outline;
  {
    size_t pts = 0;
    for (const Poly& s : shapes) pts += s.size();
    outline.reserve(pts * 2 + 4 * shapes.size());
  }
  for (const Poly& s : shapes) {  // :2015-2082
    std::vector<OutShape>& st = outline;
    const bool open = !eq(s[0], s.back());
    if (open) {
      if (lineCap == kRoundC) st.push_back(circle_shape(s[0]));
      else if (lineCap == kSquare) {
        P2 t = unit(sub(s[1], s[0]));
        st.push_back(rect_shape(sub(s[0], scl(t, hs)), s[0], hs));
      }
    }
    for (float d : dashes)
      if (d <= 0.0f) throw GeomError{"Invalid line dash value"};
    for (size_t i = 1; i < s.size(); i++) {
      P2 pos = s[i], prevPos = s[i - 1];
      if (!dashes.empty()) {
        float dist = len(sub(prevPos, pos));
        P2 dir = unit(sub(pos, prevPos));
        P2 cur = prevPos;
        bool done = false;
        while (!done) {
          for (size_t j = 0; j < dashes.size(); j++) {
            float d = dashes[j];
            if (j % 2 == 0) st.push_back(rect_shape(cur, add(cur, scl(dir, fmin_n(dist, d))), hs));
            cur = add(cur, scl(dir, d));
            dist -= d;
            if (dist <= 0) {
              done = true;
              break;
            }
          }
        }
      } else {
        st.push_back(rect_shape(prevPos, pos, hs));
      }
      if (i < s.size() - 1) join(st, prevPos, pos, s[i + 1]);
    }
    if (!open) {
      join(st, s[s.size() - 2], s.back(), s[1]);
    } else if (lineCap == kRoundC) {
      st.push_back(circle_shape(s.back()));
    } else if (lineCap == kSquare) {
      P2 t = unit(sub(s.back(), s[s.size() - 2]));
      st.push_back(rect_shape(add(s.back(), scl(t, hs)), s.back(), hs));
    }
  }
  out.reserve(out.size() + outline.size() * 5);
  for (const OutShape& o : outline) {
    if (o.circ) {
      Prim c4[4];
      circle_prims(o.c, hs, c4);
      out.insert(out.end(), c4, c4 + 4);
    } else if (o.n > 0) {  // emit_polygon_lines on the inline points
      if (!eq(o.p[o.n - 1], o.p[0])) out.push_back(line_prim(o.p[o.n - 1], o.p[0]));
      for (int i = 0; i + 1 < o.n; i++)
        if (!eq(o.p[i], o.p[i + 1])) out.push_back(line_prim(o.p[i], o.p[i + 1]));
    }
  }
}

// The polylines and per-shape parameters of a stroke for the GPU outline
// (stroke.cu); false when the stroke needs the host outline (dashes, or a
// polyline of fewer than two points).
bool build_stroke_geom(const float* cmds, int64_t n, float ps, float strokeWidth, int lineCap, int lineJoin,
                       float miterLimit, int64_t nDashes, StrokeGeom& out) {
  validate_commands(cmds, n);
  out.pts.clear();
  out.shapes.clear();
  out.nprims = 0;
  out.ncurves = 0;
  if (nDashes > 0) return false;
  const float ems = error_margin_sq(ps);
  std::vector<Poly> shapes = walk_commands(cmds, n, false, ems, nullptr);
  if (strokeWidth <= 0) return true;  // nothing to draw
  for (const Poly& s : shapes)
    if (s.size() < 2) return false;
  const StrokeCfg cfg = stroke_cfg(ps, strokeWidth, lineCap, lineJoin, miterLimit);
  const bool roundJoin = lineJoin == kRoundJ && (float)kPI * cfg.hs * cfg.hs > cfg.minArea;
  long long thr = 0;
  for (const Poly& s : shapes) {
    StrokeShape sh;
    memset(&sh, 0, sizeof sh);
    sh.pt_off = (long long)out.pts.size();
    sh.prim_off = out.nprims;
    sh.thr_off = thr;
    sh.npts = (int)s.size();
    sh.closed = eq(s[0], s.back()) ? 1 : 0;
    sh.hs = cfg.hs;
    sh.miterAngle = cfg.miterAngle;
    sh.minArea = cfg.minArea;
    sh.cap = lineCap;
    sh.join = lineJoin;
    sh.roundJoin = roundJoin ? 1 : 0;
    for (const P2& q : s) out.pts.push_back(float2{q.x, q.y});
    out.nprims += kStrokeCapSlot + (long long)kStrokeSegSlot * (sh.npts - 1);
    thr += sh.npts;
    const long long joins = sh.npts - 2 + (sh.closed ? 1 : 0);
    const long long caps = sh.closed ? 0 : 2;
    out.ncurves += 4 * ((roundJoin ? joins : 0) + (lineCap == kRoundC ? caps : 0));
    out.shapes.push_back(sh);
  }
  return true;
}

// The slot of the join at point i of a GPU-outlined shape (or, after its last
// segment, the closing join), rebuilt with the C library's atan2f, in the
// GPU outline's slot form (stroke.cu): a circle's four cubics, a polygon's
// edges in order (zero-length ones kept) padded with zero-length lines, or
// four zero-length lines.
void stroke_join_slot(const StrokeGeom& g, int shape, int i, Prim* out4) {
  const StrokeShape& sh = g.shapes[(size_t)shape];
  const float2* q = g.pts.data() + sh.pt_off;
  auto P = [&](int k) { return P2{q[k].x, q[k].y}; };
  StrokeCfg cfg;
  cfg.hs = sh.hs;
  cfg.miterAngle = sh.miterAngle;
  cfg.minArea = sh.minArea;
  cfg.cap = sh.cap;
  cfg.join = sh.join;
  const int n = sh.npts;
  OutShape o;
  const bool any =
      i < n - 1 ? join_shape(o, P(i - 1), P(i), P(i + 1), cfg) : join_shape(o, P(n - 2), P(n - 1), P(1), cfg);
  if (any && o.circ) {
    circle_prims(o.c, sh.hs, out4);
    return;
  }
  int k = 0;
  if (any)
    for (int j = 0; j + 1 < o.n; j++) out4[k++] = line_prim(o.p[j], o.p[j + 1]);
  for (; k < 4; k++) out4[k] = line_prim(P2{0, 0}, P2{0, 0});
}

float pixel_scale(const float* m) {  // paths.nim:61-66
  return fmax_n(sqrtf(m[0] * m[0] + m[1] * m[1]), sqrtf(m[3] * m[3] + m[4] * m[4]));
}
bool is_identity(const float* m) {
  static const float I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 9; i++)
    if (!(m[i] == I[i])) return false;
  return true;
}
float error_margin_sq(float ps) { return powf(kMargin / ps, 2); }  // :667

// chroma Color -> ColorRGBX: round(c*255) per channel, then premultiply with
// (c*a+127) div 255 (pinned by tests/test_images_draw.nim:282 and
// tests/test_images.nim:204-228).
uint32_t color_to_rgbx(const float* c) {
  uint32_t v[4];
  for (int i = 0; i < 4; i++) {
    float r = roundf(c[i] * 255.0f);
    v[i] = !(r > 0.0f) ? 0u : (r > 255.0f ? 255u : (uint32_t)r);
  }
  if (v[3] != 255)
    for (int i = 0; i < 3; i++) v[i] = (v[i] * v[3] + 127) / 255;
  return v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24);
}

// gaussianKernel  internal.nim:17-34 (the `1 / sqrt(2*PI*s^2) * exp(..)`
// term meets the float64 PI and is float64; `total` is float64).  Writes
// 2*radius+1 weights into `out`, using `floats` (same length) as work space;
// allocates nothing.
void gaussian_kernel_into(int64_t radius, float* f, uint16_t* out) {
  const size_t n = (size_t)(radius * 2 + 1);
  double total = 0.0;
  for (int64_t step = -radius; step <= radius; step++) {
    float s = (float)radius / 2.2f;
    float e = expf((-1.0f * ((float)step * (float)step)) / (2.0f * (s * s)));
    double a = 1.0 / sqrt((2 * kPI) * (double)(s * s)) * (double)e;
    f[(size_t)(step + radius)] = (float)a;
    total += a;
  }
  for (size_t i = 0; i < n; i++) {
    float v = (float)((double)f[i] / total);
    float r = roundf(v * 255 * 256);
    out[i] = (uint16_t)(uint32_t)(int32_t)r;
  }
}

std::vector<uint16_t> gaussian_kernel(int64_t radius) {
  std::vector<float> f((size_t)(radius * 2 + 1));
  std::vector<uint16_t> out(f.size());
  gaussian_kernel_into(radius, f.data(), out.data());
  return out;
}

// straightAlphaTable (internal.nim:68-74), a compile-time table in Nim and
// therefore evaluated in float64.
void straight_alpha_table(uint8_t* out) {
  for (int a = 0; a < 256; a++) {
    double mult = a > 0 ? 255.0 / (double)a : 0.0;
    for (int c = 0; c < 256; c++) {
      double v = round((double)c * mult);
      out[a * 256 + c] = (uint8_t)(v < 255.0 ? v : 255.0);
    }
  }
}

}  // namespace pxg
