// Shared host/device layout of the fill pipeline (pixie's fillShapes,
// src/pixie/paths.nim:1593-1912) on the GPU.
//
// One fill job = one call of fillShapes on one RGBX image.  The host turns the
// path commands into primitives (lines, quadratics, cubics; arcs and stroke
// outlines arrive as lines), the setup kernel (one CTA per job) flattens them
// into pixie's segments, reduces the bounds and derives the row-band
// partitions (each segment's band range, each band's entry count and
// anti-aliasing flag); the row kernel (one warp per image row) collects its
// band's entries in segment order, runs the reference's per-row decision and
// writes the pixels.
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

struct Band {  // Partition (paths.nim:33-36): entry count and flags
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
  long long prim_off;
  int nprims, winding;
  float ems;  // errorMarginSq = pow(0.2 / pixelScale, 2)  (paths.nim:667)
  int identity, mode;
  uint32_t rgbx;  // premultiplied paint colour
  float mat[9];
  int pad0;
  uint8_t* img;  // RGBX, row-major, W*H pixels
  long long W, H;
  long long row_off;  // prefix of work rows over the batch
  // outputs (setup kernel)
  int status, nseg, nb;
  uint32_t ph;
  long long seg_off, band_off;
  long long startX, startY, pathWidth, pathHeight;
};

enum ArenaCounter {
  kCtrSegs = 0, kCtrBands, kCtrOvfRows, kCtrXClears, kNumCounters
};

struct Arena {
  const Prim* prims;
  float4* segs;    // pixie's segments (at.x, at.y, to.x, to.y), at.y < to.y
  int* segw;       // winding of each segment
  uint2* segband;  // first and last band each segment falls in (partitionRange)
  long long seg_cap;
  Band* bands;
  long long band_cap;
  unsigned long long* counters;
  long long* ovf_rows;  // packed (job << 32 | y) rows whose crossings exceed the fast kernel
  long long ovf_cap;
  long long* xclears;   // (job, start, end) linear-pixel clears that reach into earlier rows
  long long xclear_cap;
};

}  // namespace pxg
