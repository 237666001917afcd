// Host-side geometry of the fill/stroke entry points: what pixie computes on
// the CPU before its scan converter runs, and what stays on the host here.
//   - the command walk of commandsToShapes (src/pixie/paths.nim:654-1057):
//     arc-free subpaths become GPU primitives (lines, quadratics, cubics,
//     flattened on the device); subpaths with arcs are flattened here
//     (cosf/sinf/acosf per step) and uploaded as lines;
//   - strokeShapes (paths.nim:1922-2082): stroke outlines are built here and
//     uploaded as lines;
//   - gaussianKernel (internal.nim:17-34) weights and chroma colour
//     conversion of the paint.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "raster.cuh"

namespace pxg {

struct GeomError {
  std::string msg;
};

// Builds the primitives of fillPath (closeSubpaths = true).  Throws GeomError.
void build_fill_prims(const float* cmds, int64_t n, float pixelScale, std::vector<Prim>& out);
// Builds the outline primitives of strokePath.  Throws GeomError.
void build_stroke_prims(const float* cmds, int64_t n, float pixelScale, float strokeWidth,
                        int lineCap, int lineJoin, float miterLimit, const float* dashes,
                        int64_t nDashes, std::vector<Prim>& out);
// A stroke prepared for the GPU outline (stroke.cu): its polylines' points
// back to back, one StrokeShape per polyline (slot offsets relative to the
// stroke's first primitive), the primitive count and how many are cubics.
struct StrokeGeom {
  std::vector<float2> pts;
  std::vector<StrokeShape> shapes;
  long long nprims = 0;
  long long ncurves = 0;
};
// Builds the polylines of strokePath for the GPU outline; false when the stroke
// needs the host outline (dashes, degenerate polylines).  Throws GeomError.
bool build_stroke_geom(const float* cmds, int64_t n, float pixelScale, float strokeWidth, int lineCap,
                       int lineJoin, float miterLimit, int64_t nDashes, StrokeGeom& out);
// The join slot (4 primitives) of point i of shape `shape`, with the C
// library's atan2f: the fix-up of a join the GPU found ambiguous.
void stroke_join_slot(const StrokeGeom& g, int shape, int i, Prim* out4);
// Validates the command stream (kinds, parameter counts, finiteness).
void validate_commands(const float* cmds, int64_t n);

float pixel_scale(const float* mat9);
bool is_identity(const float* mat9);
float error_margin_sq(float pixelScale);
uint32_t color_to_rgbx(const float* color4);  // straight float colour -> premultiplied RGBX
std::vector<uint16_t> gaussian_kernel(int64_t radius);
void gaussian_kernel_into(int64_t radius, float* work, uint16_t* out);  // no allocation
void straight_alpha_table(uint8_t* out256x256);

}  // namespace pxg
