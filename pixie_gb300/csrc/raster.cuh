// Shared host/device layout of the fill pipeline (pixie's fillShapes,
// src/pixie/paths.nim:1593-1912) on the GPU.
//
// One fill job = one call of fillShapes on one RGBX image.  The host turns the
// path commands into primitives (lines, quadratics, cubics; arcs and stroke
// outlines arrive as lines), the setup kernel (one CTA per job) flattens them
// into pixie's segments, reduces the bounds and derives the row-band
// partitions (each band's entry list in segment order, its count and
// anti-aliasing flag); the row kernel (one warp per image row) reads its
// band's entries, runs the reference's per-row decision and writes the
// pixels.
#pragma once
#include <vector_types.h>

#include <cstdint>

namespace pxg {

enum PrimKind { kPrimLine = 0, kPrimQuad = 1, kPrimCubic = 2 };

struct Prim {  // 48 bytes
  float x[4], y[4];
  int kind, pad[3];
};

struct Entry {  // PartitionEntry (paths.nim:28-31): clipped segment, line m/b, winding
  float ax, ay, bx, by, m, b;
  int w, pad;
};

struct Band {  // Partition (paths.nim:33-36): its entries' segment indices, count and flags
  long long off;  // first index in Arena::bandseg
  int count, flags;
};
enum BandFlags { kBandAA = 1, kBandTwoSpanning = 2 };

enum JobStatus {
  kOk = 0,
  kNothing = 1,            // pathWidth == 0: fillShapes returns before drawing
  kErrCubic = 2,           // "Unable to discretize cubic"
  kErrQuad = 3,            // "Unable to discretize quadratic"
  kErrIntOverflow = 4,     // "Path int overflow detected"
  kErrArenaFull = 5,       // workspace too small: grow and rerun
  kErrIterLimit = 6,       // flattening did not converge within the iteration cap
  kErrRowTooComplex = 7    // a row crosses more edges than the largest row kernel holds
};

struct PathJob {
  // inputs (host)
  const Prim* prims;  // device primitives of the job's path: prims[prim_off ..]
  long long pc_off;   // the job's slice of Arena::primcnt
  long long prim_off;
  int nprims, winding;
  float ems;  // errorMarginSq = pow(0.2 / pixelScale, 2)  (paths.nim:667)
  int identity, mode;
  uint32_t rgbx;  // premultiplied paint colour
  float mat[9];
  int group;     // lanes that flatten one curve together (1, 2, 4, 8, 16 or 32)
  int a8;        // img is an 8-bit alpha mask (white NormalBlend fills only), else RGBX
  uint8_t* img;  // RGBX or A8, row-major, W*H pixels
  long long W, H;
  long long row_off;  // prefix of row-kernel work items over the batch
  long long ri_off;     // scenes: row y of the job is Arena::rowidx[ri_off + y * ri_stride]
  long long ri_stride;
  int stroke_gpu;       // host: the primitives are a GPU-outlined stroke (scene: in its stroke region)
  int pad_;
  // outputs (setup kernel)
  int status, nseg, nb;
  uint32_t ph;
  long long seg_off, band_off;
  long long startX, startY, pathWidth, pathHeight;
};

// One polyline of a stroked path outlined on the GPU (strokeShapes,
// paths.nim:1922-2082, without dashes).  Its outline occupies a fixed slot of
// primitives: 4 for the start cap, then 8 per segment (its rectangle, then
// the join at its end point -- or, after the last segment, the closing join
// or the end cap).  Polygons become their edges in the reference's order;
// edges of zero length and unused slots are zero-length lines, which the
// setup kernel drops as horizontal, as shapesToSegments drops them.
struct StrokeShape {
  long long pt_off;    // first point of the polyline
  long long prim_off;  // first primitive of its slot
  long long thr_off;   // first thread of the outline kernel (exclusive prefix of npts)
  int npts, closed;    // npts >= 2; closed: first point == last point
  float hs, miterAngle, minArea;  // strokeWidth / 2, miterLimitToAngle(miterLimit), pixelErrorMargin / pixelScale
  int cap, join, roundJoin;       // LineCap, LineJoin; roundJoin: pi * hs^2 > minArea (the circle is drawn)
};
// Slot offset of point i of a shape: the start cap at 0, segment i at 4 + 8 (i - 1).
constexpr int kStrokeCapSlot = 4, kStrokeSegSlot = 8;

// Paths [j0, j1) of the job array painted in order onto one canvas (the
// jobs' img/W/H).  A launch may carry several runs on distinct canvases.
struct SceneRun {
  long long row_off;  // prefix of (row, slice) work items over the launch's runs
  long long W, H;
  uint8_t* img;       // the canvas (RGBX)
  long long ri_base;  // row y, path j: Arena::rowidx[ri_base + y * (j1 - j0) + j - j0]
  long long rec_off;  // recording items of the run: rec_off + (j - j0) * H + y
  int j0, j1;
};

// One mask of a batch drawn onto a page at an integer offset.
struct MaskDraw {
  long long off;  // byte offset of the mask in the batch's mask buffer
  long long x, y;
  int w, h;
};

enum ArenaCounter {
  kCtrSegs = 0, kCtrBands, kCtrOvfRows, kCtrXClears, kCtrBandSegs, kCtrRowErr, kCtrQueue,
  kCtrProg, kCtrProgFull, kCtrQueue2, kCtrCov8, kCtrPainted, kNumCounters
};

struct Arena {
  const Prim* prims;
  float4* segs;    // pixie's segments (at.x, at.y, to.x, to.y), at.y < to.y
  int* segw;       // winding of each segment
  uint2* segband;  // first and last band each segment falls in (partitionRange)
  long long seg_cap;
  Band* bands;
  long long band_cap;
  int* bandseg;    // per band, the indices (within the job) of its segments, ascending
  long long bandseg_cap;
  int* primcnt;    // per primitive: segments emitted, then their exclusive prefix
  long long primcnt_cap;
  int4* prog;          // scenes: row programs (16-byte units)
  long long prog_cap;
  int* rowidx;         // scenes: per row and job, the first unit of its program (-1: none)
  uint8_t* cov8;       // scenes: coverage bytes of rows recorded as kRecCov8
  long long cov8_cap;
  unsigned long long* counters;
  long long* ovf_rows;  // packed (job << 32 | y) rows whose crossings exceed the fast kernel
  long long ovf_cap;
  long long* xclears;   // (job, start, end) linear-pixel clears that reach into earlier rows
  long long xclear_cap;
  uint8_t* fsteps;      // fill setup: the halving level of every accepted flattening step, per group
  long long fsteps_cap; // (the second pass replays them); bytes
};

}  // namespace pxg
