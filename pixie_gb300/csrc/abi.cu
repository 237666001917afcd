// The C ABI of include/pxg.h: device context, image handles, the fill/stroke
// job runner and the image operations.  No C++ exception crosses the ABI;
// failures set a per-thread message returned by pxg_take_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <deque>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <atomic>
#include <vector>

#include "../../include/pxg.h"
#include "host_geom.h"
#include "paint.cuh"
#include "pxg_device.cuh"
#include "raster.cuh"

struct pxg_image {
  uint8_t* data;
  int64_t width, height;
  int owned;
  bool exported = false;  // pxg_image_device_ptr handed the address out: it must not change
  long long cap = 0;      // bytes allocated at data (owned images)
  cudaEvent_t copy_ev = nullptr;  // the last asynchronous upload or download of the image
  bool copy_pending = false;      // ... which no compute on the image has waited for yet
  cudaEvent_t compute_ev = nullptr;  // after the last compute call that named the image
  bool compute_set = false;
};

struct GraphCacheHolder;

// A batch of 8-bit masks: each the alpha of fillPath(color(1, 1, 1, 1)) on a
// transparent image of its own size.  Primitives are built at add time; the
// masks live in one device buffer.
struct pxg_masks {
  std::vector<pxg::Prim> prims;
  std::vector<pxg::PathJob> jobs;
  std::vector<long long> offs;  // byte offset of each mask
  long long bytes = 0;
  unsigned char* dev = nullptr;
  long long dev_cap = 0;
  bool rendered = false;
  pxg::Prim* dprims = nullptr;  // device copy of prims
  long long dcap = 0;
  bool dirty = true;
  GraphCacheHolder* graph = nullptr;
  ~pxg_masks();
};

// A recorded sequence of fillPath/strokePath calls (primitives built on the
// host at record time), painted in order by pxg_image_draw_scene.
struct pxg_scene {
  std::vector<pxg::Prim> prims;
  std::vector<pxg::PathJob> jobs;
  // strokes outlined on the GPU: their polylines (jobs with stroke_gpu index
  // the outline primitives in dstroke)
  pxg::StrokeGeom sk;
  // device copy of prims, uploaded at the first draw after a change, and the
  // outline primitives of sk, built there at the same time
  mutable pxg::Prim* dprims = nullptr;
  mutable long long dcap = 0;
  mutable pxg::Prim* dstroke = nullptr;
  mutable long long dscap = 0;
  mutable bool dirty = true;
  ~pxg_scene() {
    if (dprims) cudaFree(dprims);
    if (dstroke) cudaFree(dstroke);
  }
};

// The serving engine: render jobs (a recorded scene painted onto a fresh
// transparent canvas, then an optional blur) admitted against a device
// memory budget and advanced together, a bounded chunk of each job's paths
// per step (continuous batching: a job that arrives while others are on the
// GPU joins the next step; one that finishes leaves and frees its memory).
struct SrvJob {
  int64_t id;
  const pxg_scene* scene;
  int64_t W, H;
  int64_t blur;  // radius (0: none)
  int state;     // 0 queued, 1 active, 2 done, 3 failed
  int status;
  size_t next;   // next path of the scene
  long long bytes;
  pxg_image canvas;
  uint8_t* tmp;
  double t_submit, t_admit, t_done;
  std::string err;
};
struct pxg_server {
  long long budget = 0, used = 0;
  long long paths_per_job = 512;     // path chunk of one job in one step
  long long paths_per_step = 16384;  // paths of all jobs in one step
  int64_t next_id = 1;
  std::deque<SrvJob*> queue;
  std::vector<SrvJob*> active;
  std::map<int64_t, SrvJob*> jobs;
  std::vector<int64_t> finished;
  long long steps = 0, peak_used = 0, peak_active = 0;
  ~pxg_server();
};

namespace pxg {
__global__ void k_setup(PathJob* jobs, Arena A, int maxBands);
const void* rows_kernel(int v);
size_t rows_smem(int v);
int rows_warps(int v);
void launch_rows(int v, unsigned blocks, cudaStream_t st, PathJob* jobs, const long long* offs, int njobs,
                 const Arena& A, const uint8_t* tbl, long long items, int rpi);
__global__ void k_rows_wide(PathJob* jobs, Arena A, const uint8_t* tbl);
__global__ void k_xclears(PathJob* jobs, Arena A);
const void* scene_rec_kernel();
size_t scene_rec_smem();
int scene_rec_warps();
const void* scene_kernel();
int scene_warps();
int scene_tile();
void launch_scene_rec(unsigned blocks, cudaStream_t st, PathJob* jobs, const SceneRun* runs, int nruns,
                      long long items, const Arena& A, unsigned char* wide, long long slots);
void launch_scene(unsigned blocks, cudaStream_t st, PathJob* jobs, const SceneRun* runs, int nruns, long long items,
                  const Arena& A, const uint8_t* tbl, int sliceW);
size_t scene_wide_bytes();
size_t setup_smem(int maxBands);
int draw_masks_tiles();
void launch_draw_masks(int tile, uint32_t* page, long long W, long long H, const void* items, int n,
                       const uint8_t* masks, int mode, const uint8_t* tbl, cudaStream_t st);
size_t rows_smem_fast();
size_t rows_smem_wide();
int rows_warps_fast();
struct SmoothArgs {
  float px, py, dxx, dxy, dyx, dyy;
  float seg[4][4];
  long long yStart, yEnd;
};
void launch_minify2(const uint32_t* src, long long w, long long h, uint32_t* out, int nsm, cudaStream_t st);
void launch_magnify2(const uint32_t* src, long long w, long long h, uint32_t* out, int nsm, cudaStream_t st);
long long smooth_scratch_bytes(long long W, long long rows);
void launch_draw_smooth(uint32_t* a, long long W, long long H, const uint32_t* b, long long bw, long long bh,
                        const SmoothArgs& g, int mode, const uint8_t* tbl, void* scratch, int nsm,
                        cudaStream_t st);
void launch_draw(uint32_t* a, const uint32_t* b, long long Wa, long long Ha, long long Wb,
                 long long Hb, long long px, long long py, int mode, const uint8_t* tbl, int nsm,
                 cudaStream_t st);
void launch_fill(uint32_t* a, long long n, uint32_t c, int nsm, cudaStream_t st);
void launch_blend_pixels(int mode, const uint8_t* tbl, const uint32_t* bd, const uint32_t* src,
                         uint32_t* out, long long n, cudaStream_t st);
void launch_blur(uint32_t* img, uint32_t* tmp, long long W, long long H, int r,
                 const uint16_t* kern, uint32_t oob, int nsm, size_t maxSmem, cudaStream_t st);
void launch_spread(uint32_t* img, uint8_t* a0, uint8_t* a1, long long W, long long H, int s,
                   int nsm, cudaStream_t st);
void launch_shadow(const uint32_t* src, uint32_t* out, uint8_t* a0, uint8_t* a1, long long W,
                   long long H, long long ox, long long oy, int s, int r, const uint16_t* kern,
                   uint32_t color, int nsm, cudaStream_t st);
size_t blur_x_smem(int r);
void* blurb_kernel(bool x);
unsigned long long launch_count();
void note_launch();
size_t blur_y_smem(int r);
bool launch_blur_tc(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                    uint32_t oob, int nsm, size_t maxSmem, int* err, cudaStream_t st);
const void* tc_blur_kernel(bool x, int n);
bool launch_blur_tcp(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                     uint32_t oob, int nsm, size_t maxSmem, int* err, cudaStream_t st);
const void* tcp_blur_kernel(bool x, int n);
bool ring_blur_init(size_t* maxSmem);
bool weights_exact_f16(const uint16_t* hostKern, int r);
long long blur_scratch_bytes(long long W, long long H);
int ring_trace(int enable, long long* out, long long n);
bool launch_blur_ring(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                      bool exactF16, uint32_t oob, int nsm, size_t maxSmem, int* err, cudaStream_t st);
void launch_stroke_outline(const float2* pts, const StrokeShape* shapes, int nshapes, long long nthreads, Prim* out,
                           int2* amb, long long amb_cap, unsigned long long* amb_count, int nsm, cudaStream_t st);
bool launch_blur_small_fused(const uint32_t* in, uint32_t* out, long long W, long long H, int r,
                             const uint16_t* kern, uint32_t oob, cudaStream_t st);
bool launch_blur_small(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                       uint32_t oob, int nsm, cudaStream_t st);
constexpr int kSmallBlurMaxR = 8;  // the largest radius launch_blur_small(_fused) takes
__global__ void k_blur_x(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
__global__ void k_blur_y(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
__global__ void k_blurf_x(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
__global__ void k_blurf_y(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
}  // namespace pxg

using namespace pxg;

namespace {

// Per-thread error text in fixed buffers: setting an error allocates nothing.
thread_local char t_err[1024];
thread_local bool t_has_err = false;
thread_local char t_taken[1024];

struct ApiError {
  std::string msg;
};

void set_err(const char* m) {
  snprintf(t_err, sizeof t_err, "%s", m);
  t_has_err = true;
}
void set_err(const std::string& m) { set_err(m.c_str()); }

#define CU(x)                                                                               \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) throw ApiError{std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                                          " at " #x};                                       \
  } while (0)

template <class T>
void dev_grow(T*& p, long long& cap, long long need) {
  if (need <= cap && p) return;
  long long n = std::max(need, cap * 2);
  if (n < 1024) n = 1024;
  if (p) cudaFree(p);
  p = nullptr;
  CU(cudaMalloc((void**)&p, sizeof(T) * (size_t)n));
  cap = n;
}

struct Ctx {
  std::recursive_mutex mu;
  bool ready = false;
  int dev = 0, nsm = 0;
  size_t smemOptin = 48 * 1024;
  size_t setupSmemMax = 0, blurSmemMax = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  // Non-blocking mode: uploads and downloads run on their own streams.  Each
  // call's compute waits for the copies issued before it (copies_pending); a
  // copy waits for the compute issued before it (compute_ev, recorded at the
  // end of every call once copies went asynchronous) and for the image's own
  // previous copy (pxg_image::copy_ev).
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t compute_ev = nullptr;
  bool async_copies = false;
  std::vector<cudaEvent_t> copies_pending, ev_pool;
  uint8_t* tbl = nullptr;
  // fill arena
  float4* segs = nullptr;
  int* segw = nullptr;
  long long seg_cap = 0, segw_cap = 0;
  uint2* segband = nullptr;
  long long segband_cap = 0;
  Band* bands = nullptr;
  long long band_cap = 0;
  int* bandseg = nullptr;
  long long bandseg_cap = 0;
  int* primcnt = nullptr;
  long long primcnt_cap = 0;
  MaskDraw* mdraw = nullptr;      // mask positions of pxg_image_draw_masks
  long long mdraw_cap = 0;
  int4* prog = nullptr;           // scene row programs
  long long prog_cap = 0;
  int* rowidx = nullptr;          // scene rows -> program
  long long rowidx_cap = 0;
  uint8_t* cov8 = nullptr;        // scene coverage bytes (rows that fit; the rest keep spans)
  long long cov8_cap = 0;
  unsigned char* wide = nullptr;  // per-warp wide row scratch of the scene recording kernel
  long long wide_slots = 0;
  long long* ovf = nullptr;
  long long ovf_cap = 0;
  long long* xcl = nullptr;
  long long xcl_cap = 0;
  uint32_t* pt_buf[2] = {nullptr, nullptr};  // the mask and the fill image of a non-solid paint
  long long pt_cap[2] = {0, 0};
  float* pt_stops = nullptr;  // gradient stops on the device
  long long pt_stops_cap = 0;
  uint32_t* sm_buf[2] = {nullptr, nullptr};  // minify/magnify pre-pass images (ping-pong)
  long long sm_cap[2] = {0, 0};
  uint8_t* fsteps = nullptr;  // flattening step records (fill setup)
  long long fsteps_cap = 0;
  // upload area: jobs | counters | prims (device and pinned mirror)
  unsigned char* d_up = nullptr;
  unsigned char* h_up = nullptr;
  size_t up_cap = 0;
  // misc scratch
  uint16_t* kern = nullptr;
  long long kern_cap = 0;
  unsigned char* scratch = nullptr;
  long long scratch_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evr0 = nullptr, evr1 = nullptr;
  int* dev_err = nullptr;   // device-side error flag (a tensor-core wait that ran out)
  int* host_err = nullptr;  // its pinned mirror
  // blur kernels: 3 register-blocked CUDA-core passes for radii up to 8, TMA-fed ring passes on the
  // tensor cores above (falling back to 1, then 0, where they do not apply), 1 pipelined
  // tensor-core passes, 2 single-stage ones, 0 the tiled CUDA-core passes
  int blur_tensor = 3;
  size_t tcSmemMax = 0;
  bool ring_ok = false;  // the ring kernels and the driver's tensor-map encoder are available
  int last_blur = -1;    // kernel family of the last blur (4: the small-radius passes)
  size_t ringSmemMax = 0;
  float last_ms = 0;
  long long stats[6] = {0, 0, 0, 0, 0, 0};  // last fill launch: paths, prims, segments, entries, blends, wide rows
  int rows_ctas_per_sm[2] = {1, 1};  // resident CTAs of each row-kernel variant
  int scene_ctas_per_sm[2] = {1, 1};  // resident CTAs of the scene recording and drawing kernels
  int scene_slice = 256;              // pixels of a row one warp of the drawing pass owns (0: chosen per launch)
  bool stroke_gpu = true;             // outline strokes without dashes on the GPU (stroke.cu)
  float2* sk_pts = nullptr;           // outline kernel inputs: polyline points, shapes
  long long sk_pts_cap = 0;
  StrokeShape* sk_shapes = nullptr;
  long long sk_shapes_cap = 0;
  int2* sk_amb = nullptr;             // joins the outline kernel found ambiguous
  long long sk_amb_cap = 0;
  unsigned long long* sk_ambn = nullptr;
  Prim* sk_prims = nullptr;           // the outline of a single strokePath call
  long long sk_prims_cap = 0;
  long long sk_fixups = 0;            // ambiguous joins rebuilt on the host (all calls)
  bool blocking = true;  // image operations wait for their GPU work
  std::map<int64_t, uint16_t*> weights;  // gaussian weights per radius, on the device
  std::map<int64_t, bool> weights_f16;   // every weight of the radius is an exact f16
};
Ctx g;

// Lets a kernel use all the opt-in shared memory left after its static part.
size_t allow_max_smem(const void* fn) {
  cudaFuncAttributes fa;
  CU(cudaFuncGetAttributes(&fa, fn));
  size_t dyn = g.smemOptin > fa.sharedSizeBytes ? g.smemOptin - fa.sharedSizeBytes : 0;
  CU(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  return dyn;
}

void init_locked(int device) {
  if (g.ready) return;
  CU(cudaSetDevice(device));
  cudaDeviceProp prop;
  CU(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) throw ApiError{"pxg requires a Blackwell-class GPU (sm_103a build)"};
  g.dev = device;
  g.nsm = prop.multiProcessorCount;
  g.smemOptin = prop.sharedMemPerBlockOptin;
  CU(cudaStreamCreateWithFlags(&g.own, cudaStreamNonBlocking));
  g.stream = g.own;
  CU(cudaStreamCreateWithFlags(&g.h2d, cudaStreamNonBlocking));
  CU(cudaStreamCreateWithFlags(&g.d2h, cudaStreamNonBlocking));
  CU(cudaEventCreateWithFlags(&g.compute_ev, cudaEventDisableTiming));
  // the straight-alpha table (256 x 256 bytes), then v / 255.0f for
  // v = 0..255, then SoftLight's D of that value (W3C: ((16 cb - 12) cb + 4) cb
  // for cb <= 0.25, else sqrt(cb); float operations in this order, uncontracted)
  std::vector<uint8_t> t(kTblBytes);
  straight_alpha_table(t.data());
  for (int v = 0; v < 256; v++) {
    const float f = (float)v / 255.0f;
    memcpy(t.data() + kTblUnitOff + 4 * v, &f, 4);
    const float d = f <= 0.25f ? ((16.0f * f - 12.0f) * f + 4.0f) * f : sqrtf(f);
    memcpy(t.data() + kTblSoftOff + 4 * v, &d, 4);
  }
  CU(cudaMalloc(&g.tbl, kTblBytes));
  CU(cudaMemcpy(g.tbl, t.data(), kTblBytes, cudaMemcpyHostToDevice));
  for (int v = 0; v < 2; v++) {
    CU(cudaFuncSetAttribute(rows_kernel(v), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem(v)));
    int per = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, rows_kernel(v), rows_warps(v) * 32, rows_smem(v)));
    g.rows_ctas_per_sm[v] = std::max(1, per);
  }
  CU(cudaFuncSetAttribute(k_rows_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem_wide()));
  {
    CU(cudaFuncSetAttribute(scene_rec_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scene_rec_smem()));
    int per = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, scene_rec_kernel(), scene_rec_warps() * 32,
                                                     scene_rec_smem()));
    g.scene_ctas_per_sm[0] = std::max(1, per);
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, scene_kernel(), scene_warps() * 32, 0));
    g.scene_ctas_per_sm[1] = std::max(1, per);
  }
  g.setupSmemMax = allow_max_smem((const void*)k_setup);
  g.blurSmemMax = std::min(allow_max_smem((const void*)k_blur_x), allow_max_smem((const void*)k_blur_y));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem((const void*)k_blurf_x));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem((const void*)k_blurf_y));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem(blurb_kernel(true)));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem(blurb_kernel(false)));
  CU(cudaEventCreate(&g.ev0));
  CU(cudaEventCreate(&g.ev1));
  CU(cudaEventCreate(&g.evr0));
  CU(cudaEventCreate(&g.evr1));
  CU(cudaMalloc(&g.dev_err, sizeof(int)));
  CU(cudaMemset(g.dev_err, 0, sizeof(int)));
  CU(cudaMallocHost(&g.host_err, sizeof(int)));
  *g.host_err = 0;
  g.tcSmemMax = allow_max_smem(tc_blur_kernel(true, 128));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tc_blur_kernel(false, 128)));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tc_blur_kernel(true, 64)));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tc_blur_kernel(false, 64)));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tcp_blur_kernel(true, 64)));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tcp_blur_kernel(false, 64)));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tcp_blur_kernel(true, 32)));
  g.tcSmemMax = std::min(g.tcSmemMax, allow_max_smem(tcp_blur_kernel(false, 32)));
  g.ring_ok = ring_blur_init(&g.ringSmemMax);
  g.ready = true;
}
void ensure_init() {
  if (!g.ready) init_locked(0);
}

// gaussianKernel(radius) uploaded once per radius (internal.nim:17-34)
const uint16_t* weights_for(int64_t r) {
  auto it = g.weights.find(r);
  if (it != g.weights.end()) return it->second;
  std::vector<uint16_t> k = gaussian_kernel(r);
  uint16_t* d = nullptr;
  CU(cudaMalloc((void**)&d, k.size() * 2));
  CU(cudaMemcpy(d, k.data(), k.size() * 2, cudaMemcpyHostToDevice));
  g.weights[r] = d;
  g.weights_f16[r] = r <= (1 << 16) && weights_exact_f16(k.data(), (int)r);
  return d;
}

// Both blur passes of an RGBX image (img -> tmp -> img) with the configured
// kernels; a kernel family that does not take this image or radius hands it
// to the next one.  With swap_ok the caller owns both buffers and lets the
// result land in tmp: radii 1..8 then run as one fused launch (img -> tmp)
// and the function returns true, after which the caller exchanges the two
// buffers.
// tmp holds tmp_bytes: W * H * 4 at least; the tensor-core passes need
// blur_scratch_bytes(W, H) (a padded intermediate) and are skipped below that.
bool blur_dispatch(uint32_t* img, uint32_t* tmp, long long tmp_bytes, long long W, long long H, int64_t r,
                   uint32_t oob, bool swap_ok = false) {
  const uint16_t* kern = weights_for(r);
  if (swap_ok && g.blur_tensor == 3 && launch_blur_small_fused(img, tmp, W, H, (int)r, kern, oob, g.stream)) {
    g.last_blur = 5;
    return true;
  }
  int used = -1;
  if (g.blur_tensor == 3 && launch_blur_small(img, tmp, W, H, (int)r, kern, oob, g.nsm, g.stream)) used = 4;
  if (used < 0 && g.blur_tensor == 3 && g.ring_ok && tmp_bytes >= blur_scratch_bytes(W, H) &&
      launch_blur_ring(img, tmp, W, H, (int)r, kern, g.weights_f16[r], oob, g.nsm, g.ringSmemMax, g.dev_err,
                       g.stream))
    used = 3;
  if (used < 0 && g.blur_tensor == 2 &&
      launch_blur_tc(img, tmp, W, H, (int)r, kern, oob, g.nsm, g.tcSmemMax, g.dev_err, g.stream))
    used = 2;
  if (used < 0 && (g.blur_tensor == 1 || g.blur_tensor == 3) &&
      launch_blur_tcp(img, tmp, W, H, (int)r, kern, oob, g.nsm, g.tcSmemMax, g.dev_err, g.stream))
    used = 1;
  if (used < 0) {
    launch_blur(img, tmp, W, H, (int)r, kern, oob, g.nsm, g.blurSmemMax, g.stream);
    used = 0;
  }
  g.last_blur = used;
  return false;
}

void* scratch(long long bytes) {
  dev_grow(g.scratch, g.scratch_cap, bytes);
  return g.scratch;
}

struct Timed {
  bool force;
  explicit Timed(bool f = false) : force(f) {
    if (g.blocking || force) cudaEventRecord(g.ev0, g.stream);
  }
  void done() {
    if (!(g.blocking || force)) return;
    cudaEventRecord(g.ev1, g.stream);
    CU(cudaEventSynchronize(g.ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, g.ev0, g.ev1);
    g.last_ms = ms;
  }
};

// Reads (and clears) the device error flag; throws if a kernel reported a
// wait that ran out.
void check_device_error() {
  CU(cudaMemcpyAsync(g.host_err, g.dev_err, sizeof(int), cudaMemcpyDeviceToHost, g.stream));
  CU(cudaStreamSynchronize(g.stream));
  if (*g.host_err) {
    *g.host_err = 0;
    CU(cudaMemsetAsync(g.dev_err, 0, sizeof(int), g.stream));
    throw ApiError{"GPU wait timed out (tensor-core blur)"};
  }
}

const char* status_message(int st) {
  switch (st) {
    case kErrCubic: return "Unable to discretize cubic";
    case kErrQuad: return "Unable to discretize quadratic";
    case kErrIntOverflow: return "Path int overflow detected";
    case kErrIterLimit: return "Unable to discretize: flattening did not converge";
    case kErrRowTooComplex: return "Path too complex: a scanline crosses more than 4096 edges";
    case kErrArenaFull: return "Out of workspace memory";
  }
  return "Unknown error";
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Nim's round(v).int: half away from zero; out of range -> INT64_MIN
int64_t nim_round_int(float v) {
  float r = roundf(v);
  if (!(r >= -9223372036854775808.0f && r < 9223372036854775808.0f)) return INT64_MIN;
  return (int64_t)r;
}

// Lanes per curve in the setup kernel's flattening: the 256 threads of a job's
// CTA shared out over its curves (a power of two, 1..32).
int curve_group(const std::vector<Prim>& prims, long long off, int n) {
  long long curves = 0;
  for (int i = 0; i < n; i++) curves += prims[(size_t)(off + i)].kind != kPrimLine;
  int gsz = 1;
  while (gsz < 32 && curves * gsz * 2 <= 256) gsz *= 2;
  return gsz;
}

// Workspace of the fill kernels, grown on demand (never shrunk).
void ensure_arena(long long seg_need, long long list_need, long long nbands, long long nprims, long long rows) {
  dev_grow(g.segs, g.seg_cap, seg_need);
  dev_grow(g.segw, g.segw_cap, g.seg_cap);
  dev_grow(g.segband, g.segband_cap, g.seg_cap);
  dev_grow(g.bands, g.band_cap, nbands);
  dev_grow(g.bandseg, g.bandseg_cap, list_need);
  dev_grow(g.primcnt, g.primcnt_cap, nprims + 1);
  dev_grow(g.ovf, g.ovf_cap, rows);
  dev_grow(g.xcl, g.xcl_cap, 3 * (2 * rows + 1024));
}

// One host->device copy of jobs | counters | extra | prims through the pinned
// upload area.
struct Staged {
  PathJob* dj;
  unsigned char* extra;
  size_t jobsBytes, ctrBytes, extraBytes, upBytes;
  Arena A;
};
Staged stage(const std::vector<PathJob>& run, const void* extra, size_t extraBytes,
             const std::vector<Prim>& prims, bool copy = true) {
  Staged S;
  const size_t nr = run.size();
  S.jobsBytes = align_up(sizeof(PathJob) * std::max<size_t>(nr, 1), 256);
  S.ctrBytes = 256;
  S.extraBytes = align_up(extraBytes, 256);
  const size_t primBytes = sizeof(Prim) * std::max<size_t>(prims.size(), 1);
  const size_t need = S.jobsBytes + S.ctrBytes + S.extraBytes + primBytes;
  if (need > g.up_cap) {
    CU(cudaStreamSynchronize(g.stream));  // the old area may still be in flight
    if (g.d_up) cudaFree(g.d_up);
    if (g.h_up) cudaFreeHost(g.h_up);
    g.d_up = nullptr;
    g.h_up = nullptr;
    size_t cap = std::max(need, g.up_cap * 2);
    CU(cudaMalloc(&g.d_up, cap));
    CU(cudaMallocHost(&g.h_up, cap));
    g.up_cap = cap;
  }
  if (nr) memcpy(g.h_up, run.data(), sizeof(PathJob) * nr);
  {  // jobs without resident primitives read the staged ones
    const size_t primAt0 = S.jobsBytes + S.ctrBytes + S.extraBytes;
    PathJob* hj = reinterpret_cast<PathJob*>(g.h_up);
    for (size_t i = 0; i < nr; i++)
      if (!hj[i].prims) hj[i].prims = reinterpret_cast<const Prim*>(g.d_up + primAt0);
  }
  unsigned long long* hc = reinterpret_cast<unsigned long long*>(g.h_up + S.jobsBytes);
  memset(hc, 0, S.ctrBytes);
  hc[kCtrRowErr] = ~0ull;
  if (extraBytes) memcpy(g.h_up + S.jobsBytes + S.ctrBytes, extra, extraBytes);
  const size_t primAt = S.jobsBytes + S.ctrBytes + S.extraBytes;
  if (!prims.empty()) memcpy(g.h_up + primAt, prims.data(), sizeof(Prim) * prims.size());
  S.upBytes = need;
  if (copy) CU(cudaMemcpyAsync(g.d_up, g.h_up, need, cudaMemcpyHostToDevice, g.stream));
  S.dj = reinterpret_cast<PathJob*>(g.d_up);
  S.extra = g.d_up + S.jobsBytes + S.ctrBytes;
  Arena& A = S.A;
  A.prims = reinterpret_cast<const Prim*>(g.d_up + primAt);
  A.segs = g.segs;
  A.segw = g.segw;
  A.seg_cap = g.seg_cap;
  A.segband = g.segband;
  A.bands = g.bands;
  A.band_cap = g.band_cap;
  A.bandseg = g.bandseg;
  A.bandseg_cap = g.bandseg_cap;
  A.primcnt = g.primcnt;
  A.primcnt_cap = g.primcnt_cap;
  A.prog = g.prog;
  A.prog_cap = g.prog_cap;
  A.rowidx = g.rowidx;
  A.cov8 = g.cov8;
  A.cov8_cap = g.cov8_cap;
  A.counters = reinterpret_cast<unsigned long long*>(g.d_up + S.jobsBytes);
  A.ovf_rows = g.ovf;
  A.ovf_cap = g.ovf_cap;
  A.xclears = g.xcl;
  A.xclear_cap = g.xcl_cap / 3;
  if (!g.fsteps) {  // step records of the first 16 setup CTAs of a launch (512 steps x 256 groups each)
    CU(cudaMalloc(&g.fsteps, (size_t)16 * 256 * 512));
    g.fsteps_cap = (long long)16 * 256 * 512;
  }
  A.fsteps = g.fsteps;
  A.fsteps_cap = g.fsteps_cap;
  return S;
}

void note_stats(long long paths, long long prims, const unsigned long long* ctr) {
  g.stats[0] = paths;
  g.stats[1] = prims;
  g.stats[2] = (long long)ctr[kCtrSegs];
  g.stats[3] = (long long)ctr[kCtrBandSegs];
  g.stats[4] = (long long)ctr[kCtrPainted];
  g.stats[5] = (long long)ctr[kCtrOvfRows];
}

int setup_max_bands(long long maxH) {
  const int maxBands = (int)(std::max<long long>(1, maxH / 4) + 1);
  if (setup_smem(maxBands) > g.setupSmemMax) throw ApiError{"Image too tall for the fill kernels"};
  return maxBands;
}

// Grows the workspace after a launch in which some job ran out of it.
void grow_needs(const unsigned long long* ctr, long long& seg_need, long long& list_need) {
  seg_need = std::max<long long>(seg_need, (long long)ctr[kCtrSegs] * 2);
  list_need = std::max<long long>(list_need, (long long)ctr[kCtrBandSegs] * 2);
  if ((long long)ctr[kCtrSegs] <= g.seg_cap && (long long)ctr[kCtrBandSegs] <= g.bandseg_cap) {
    seg_need *= 2;
    list_need *= 2;
  }
}

// Runs fill jobs whose primitives are already in `prims` (job.prim_off set).
// Jobs must target distinct images: a job whose workspace ran out is rerun
// alone, after the others were drawn.  Returns per-job status.
// Row-kernel configuration of a fill launch: scratch variant and rows per
// work item.
struct RowsCfg {
  int variant = 0;
  int rpi = 1;
};

// A captured launch sequence (upload, setup, rows, status read-back), replayed
// while the launch's shape and buffers are unchanged.
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  std::vector<long long> key;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key.clear();
  }
};

struct RunOpts {
  RowsCfg cfg;
  unsigned char* zero = nullptr;  // buffer cleared before the first launch (mask batches)
  long long zero_bytes = 0;
  GraphCache* graph = nullptr;    // capture / replay the first launch
  float* rows_ms = nullptr;       // row-kernel time of the first launch (autotuning)
  const Prim* dprims = nullptr;   // primitives already on the device (else staged)
  long long ndprims = -1;         // how many, when `prims` does not hold them (a GPU outline)
};

// Runs fill jobs whose primitives are already in `prims` (job.prim_off set).
// Jobs must target distinct images: a job whose workspace ran out is rerun
// alone, after the others were drawn.  Returns per-job status.
void run_jobs(std::vector<PathJob>& jobs, const std::vector<Prim>& prims, std::vector<int>& status,
              const RunOpts& opts = RunOpts()) {
  const RowsCfg cfg = opts.cfg;
  const int nj = (int)jobs.size();
  status.assign((size_t)nj, kOk);
  std::vector<int> todo(nj);
  for (int i = 0; i < nj; i++) todo[i] = i;
  const long long nprims = opts.dprims && opts.ndprims >= 0 ? opts.ndprims : (long long)prims.size();
  long long seg_need = std::max<long long>(1 << 16, nprims * 8);
  long long list_need = seg_need * 4;
  for (int attempt = 0; attempt < 12 && !todo.empty(); attempt++) {
    std::vector<PathJob> run;
    long long rows = 0, maxH = 1;
    long long items = 0;
    for (int i : todo) {
      PathJob j = jobs[i];
      if (j.group == 0) j.group = curve_group(prims, j.prim_off, j.nprims);
      j.pc_off = j.prim_off;
      if (!opts.dprims) j.prims = nullptr;  // the staged copy
      else j.prims = opts.dprims;
      j.row_off = items;
      items += (j.H + cfg.rpi - 1) / cfg.rpi;
      rows += j.H;
      maxH = std::max<long long>(maxH, j.H);
      j.status = kOk;
      run.push_back(j);
    }
    const int nr = (int)run.size();
    const int maxBands = setup_max_bands(maxH);
    ensure_arena(seg_need, list_need, (long long)nr * maxBands, nprims, rows);
    const bool graphed = opts.graph && attempt == 0 && g.stream != nullptr;
    std::vector<long long> offs((size_t)nr);
    for (int r = 0; r < nr; r++) offs[(size_t)r] = run[(size_t)r].row_off;
    Staged S = stage(run, offs.data(), sizeof(long long) * offs.size(), opts.dprims ? std::vector<Prim>() : prims,
                     false);
    Arena& A = S.A;
    PathJob* dj = S.dj;
    const int v = cfg.variant;
    long long blocks = (items + rows_warps(v) - 1) / rows_warps(v);
    blocks = std::min<long long>(blocks, (long long)g.nsm * g.rows_ctas_per_sm[v]);
    blocks = std::max<long long>(blocks, 1);
    const bool timeRows = opts.rows_ms && attempt == 0 && !graphed;
    auto issue = [&](bool count) {
      if (attempt == 0 && opts.zero) CU(cudaMemsetAsync(opts.zero, 0, (size_t)opts.zero_bytes, g.stream));
      CU(cudaMemcpyAsync(g.d_up, g.h_up, S.upBytes, cudaMemcpyHostToDevice, g.stream));
      k_setup<<<nr, 256, setup_smem(maxBands), g.stream>>>(dj, A, maxBands);
      if (count) note_launch();
      CU(cudaGetLastError());
      if (timeRows) CU(cudaEventRecord(g.evr0, g.stream));
      launch_rows(v, (unsigned)blocks, g.stream, dj, reinterpret_cast<const long long*>(S.extra), nr, A, g.tbl, items,
                  cfg.rpi);
      if (count) note_launch();
      CU(cudaGetLastError());
      if (timeRows) CU(cudaEventRecord(g.evr1, g.stream));
      CU(cudaMemcpyAsync(g.h_up, g.d_up, S.jobsBytes + S.ctrBytes, cudaMemcpyDeviceToHost, g.stream));
    };
    if (graphed) {
      std::vector<long long> key = {nr, items, (long long)S.upBytes, (long long)(uintptr_t)g.d_up,
                                    (long long)(uintptr_t)g.h_up, (long long)(uintptr_t)g.segs, g.seg_cap,
                                    (long long)(uintptr_t)g.bandseg, g.bandseg_cap,
                                    (long long)(uintptr_t)g.bands, g.band_cap, (long long)(uintptr_t)g.primcnt,
                                    g.primcnt_cap, (long long)(uintptr_t)g.ovf, g.ovf_cap,
                                    (long long)(uintptr_t)g.xcl, g.xcl_cap, v, cfg.rpi, blocks, maxBands,
                                    (long long)(uintptr_t)opts.zero, opts.zero_bytes,
                                    (long long)(uintptr_t)g.stream, (long long)(uintptr_t)opts.dprims};
      GraphCache& gc = *opts.graph;
      if (!gc.exec || gc.key != key) {
        gc.reset();
        CU(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
        try {
          issue(false);
        } catch (...) {
          cudaGraph_t gr = nullptr;
          cudaStreamEndCapture(g.stream, &gr);
          if (gr) cudaGraphDestroy(gr);
          throw;
        }
        cudaGraph_t gr = nullptr;
        CU(cudaStreamEndCapture(g.stream, &gr));
        cudaError_t e = cudaGraphInstantiate(&gc.exec, gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) {
          gc.exec = nullptr;
          CU(e);
        }
        gc.key = key;
      }
      CU(cudaGraphLaunch(gc.exec, g.stream));
      note_launch();
      note_launch();
    } else {
      issue(true);
    }
    CU(cudaStreamSynchronize(g.stream));
    if (timeRows) CU(cudaEventElapsedTime(opts.rows_ms, g.evr0, g.evr1));
    unsigned long long ctr[kNumCounters];
    memcpy(ctr, g.h_up + S.jobsBytes, sizeof ctr);
    note_stats(nr, nprims, ctr);
    if (ctr[kCtrOvfRows] > 0 || ctr[kCtrXClears] > 0) {
      if ((long long)ctr[kCtrXClears] > A.xclear_cap) throw ApiError{"Out of workspace memory (cross-row clears)"};
      if (ctr[kCtrOvfRows] > 0) {
        long long b = std::min<long long>((long long)ctr[kCtrOvfRows], (long long)g.nsm * 4);
        k_rows_wide<<<(unsigned)b, 32, rows_smem_wide(), g.stream>>>(dj, A, g.tbl); note_launch();
        CU(cudaGetLastError());
      }
      if (ctr[kCtrXClears] > 0) {
        long long b = std::min<long long>((long long)ctr[kCtrXClears], 4096);
        k_xclears<<<(unsigned)b, 256, 0, g.stream>>>(dj, A); note_launch();
        CU(cudaGetLastError());
      }
      CU(cudaMemcpyAsync(g.h_up, g.d_up, S.jobsBytes, cudaMemcpyDeviceToHost, g.stream));
      CU(cudaStreamSynchronize(g.stream));
    }
    const PathJob* out = reinterpret_cast<const PathJob*>(g.h_up);
    std::vector<int> again;
    bool grow = false;
    for (int r = 0; r < nr; r++) {
      int st = out[r].status;
      int i = todo[(size_t)r];
      jobs[(size_t)i] = out[r];
      if (st == kErrArenaFull) {
        again.push_back(i);
        grow = true;
      } else {
        status[(size_t)i] = st == kNothing ? kOk : st;
      }
    }
    if (grow) grow_needs(ctr, seg_need, list_need);
    todo = again;
  }
  for (int i : todo) status[(size_t)i] = kErrArenaFull;
}

// A run of paths painted in order onto one canvas (a scene, or one serving
// job's chunk of paths).
struct HostRun {
  pxg_image* canvas;
  std::vector<PathJob>* jobs;  // the run's paths, in order; img/W/H are set here
  const std::vector<Prim>* prims;  // host primitives (jobs' prim_off index them)
  const Prim* dprims;              // the same primitives on the device
  size_t j0, j1;               // paths still to paint
  int status;                  // first failure (kOk when every path was painted)
  const Prim* dstroke = nullptr;   // GPU-outlined strokes' primitives (jobs with stroke_gpu)
};

// Lanes per curve of a path with `curves` curve primitives (curve_group).
int group_for(long long curves) {
  int gsz = 1;
  while (gsz < 32 && curves * gsz * 2 <= 256) gsz *= 2;
  return gsz;
}

// Builds the outline primitives of sg into dout (stroke.cu): uploads the
// polylines, runs the outline kernel, then rebuilds on the host, with the C
// library's atan2f, every join whose decision the kernel found ambiguous and
// writes those slots over the kernel's.  Waits for the GPU.
void outline_strokes(const StrokeGeom& sg, Prim* dout) {
  if (sg.shapes.empty() || sg.nprims == 0) return;
  const long long npts = (long long)sg.pts.size(), nsh = (long long)sg.shapes.size();
  dev_grow(g.sk_pts, g.sk_pts_cap, npts);
  dev_grow(g.sk_shapes, g.sk_shapes_cap, nsh);
  dev_grow(g.sk_amb, g.sk_amb_cap, npts);
  if (!g.sk_ambn) CU(cudaMalloc(&g.sk_ambn, sizeof(unsigned long long)));
  CU(cudaMemcpyAsync(g.sk_pts, sg.pts.data(), sizeof(float2) * (size_t)npts, cudaMemcpyHostToDevice, g.stream));
  CU(cudaMemcpyAsync(g.sk_shapes, sg.shapes.data(), sizeof(StrokeShape) * (size_t)nsh, cudaMemcpyHostToDevice,
                     g.stream));
  CU(cudaMemsetAsync(g.sk_ambn, 0, sizeof(unsigned long long), g.stream));
  launch_stroke_outline(g.sk_pts, g.sk_shapes, (int)nsh, npts, dout, g.sk_amb, npts, g.sk_ambn, g.nsm, g.stream);
  CU(cudaGetLastError());
  unsigned long long namb = 0;
  CU(cudaMemcpyAsync(&namb, g.sk_ambn, sizeof namb, cudaMemcpyDeviceToHost, g.stream));
  CU(cudaStreamSynchronize(g.stream));
  if (namb == 0) return;
  const long long n = std::min<long long>((long long)namb, npts);
  std::vector<int2> amb((size_t)n);
  CU(cudaMemcpy(amb.data(), g.sk_amb, sizeof(int2) * (size_t)n, cudaMemcpyDeviceToHost));
  std::vector<Prim> fix((size_t)n * 4);
  for (long long k = 0; k < n; k++) {
    const StrokeShape& sh = sg.shapes[(size_t)amb[(size_t)k].x];
    const int i = amb[(size_t)k].y;
    stroke_join_slot(sg, amb[(size_t)k].x, i, &fix[(size_t)k * 4]);
    const long long at = sh.prim_off + kStrokeCapSlot + (long long)kStrokeSegSlot * (i - 1) + 4;
    CU(cudaMemcpyAsync(dout + at, &fix[(size_t)k * 4], sizeof(Prim) * 4, cudaMemcpyHostToDevice, g.stream));
  }
  CU(cudaStreamSynchronize(g.stream));
  g.sk_fixups += n;
}

// Appends a GPU-outlined stroke to a scene's stroke set: its shapes' point,
// primitive and thread offsets move past the ones already there.  Returns the
// stroke's first primitive in the scene's stroke region.
long long append_stroke(StrokeGeom& dst, const StrokeGeom& src) {
  const long long p0 = (long long)dst.pts.size(), prim0 = dst.nprims;
  const long long t0 = dst.shapes.empty() ? 0 : dst.shapes.back().thr_off + dst.shapes.back().npts;
  dst.pts.insert(dst.pts.end(), src.pts.begin(), src.pts.end());
  for (StrokeShape sh : src.shapes) {
    sh.pt_off += p0;
    sh.prim_off += prim0;
    sh.thr_off += t0;
    dst.shapes.push_back(sh);
  }
  dst.nprims += src.nprims;
  dst.ncurves += src.ncurves;
  return prim0;
}

// The scene's primitives on the device, uploaded once after each change.
const Prim* scene_device_prims(const pxg_scene* sc) {
  if (sc->dirty) {
    dev_grow(sc->dprims, sc->dcap, std::max<long long>((long long)sc->prims.size(), 1));
    if (!sc->prims.empty())
      CU(cudaMemcpy(sc->dprims, sc->prims.data(), sizeof(Prim) * sc->prims.size(), cudaMemcpyHostToDevice));
    if (sc->sk.nprims > 0) {
      dev_grow(sc->dstroke, sc->dscap, sc->sk.nprims);
      outline_strokes(sc->sk, sc->dstroke);
    }
    sc->dirty = false;
  }
  return sc->dprims;
}

// The row slice of the drawing pass.  Each work item replays every path of
// its run, so items are long and the kernel lasts as long as its busiest
// warp: the slice is chosen so that the launch has about three items per
// resident warp (at most 256 pixels, the shared-memory stage), unless a
// width was set with pxg_scene_config.
int scene_slice_for(const std::vector<HostRun>& runs) {
  if (g.scene_slice > 0) return g.scene_slice;
  long long rows = 0, wmax = 1;
  for (const HostRun& r : runs) {
    if (r.status != kOk || r.j0 >= r.j1) continue;
    rows += r.canvas->height;
    wmax = std::max<long long>(wmax, r.canvas->width);
  }
  const long long slots = (long long)g.nsm * g.scene_ctas_per_sm[1] * scene_warps();
  const long long per_row = std::max<long long>(1, (3 * slots + rows - 1) / std::max<long long>(rows, 1));
  long long w = (wmax + per_row - 1) / per_row;
  w = std::max<long long>(32, std::min<long long>(w, scene_tile()));
  return (int)w;
}

// Paints several runs (distinct canvases) in one setup + scene launch pair,
// repeating for runs whose workspace ran out.  MaskBlend paths must not be
// inside a run (their clears reach outside the rows the run owns).
void run_scene_runs(std::vector<HostRun>& runs) {
  long long prim_total = 0;  // primitives of the paths this launch draws
  for (auto& r : runs)
    for (size_t j = r.j0; j < r.j1; j++) prim_total += (*r.jobs)[j].nprims;
  long long seg_need = std::max<long long>(1 << 16, prim_total * 4);
  long long list_need = seg_need * 4;
  long long prog_need = 0;
  for (auto& r : runs) r.status = kOk;
  for (int attempt = 0; attempt < 16; attempt++) {
    std::vector<PathJob> dev;
    long long pc = 0;
    std::vector<SceneRun> sr;
    std::vector<size_t> which;  // launch run -> runs index
    long long items = 0, recItems = 0, riTotal = 0, maxH = 1;
    const int slice = scene_slice_for(runs);
    for (size_t ri = 0; ri < runs.size(); ri++) {
      HostRun& r = runs[ri];
      if (r.status != kOk || r.j0 >= r.j1) continue;
      SceneRun s;
      s.row_off = items;
      s.W = r.canvas->width;
      s.H = r.canvas->height;
      s.img = r.canvas->data;
      s.j0 = (int)dev.size();
      s.ri_base = riTotal;
      s.rec_off = recItems;
      const long long nrun = (long long)(r.j1 - r.j0);
      for (size_t j = r.j0; j < r.j1; j++) {
        PathJob pj = (*r.jobs)[j];
        if (pj.group == 0) pj.group = curve_group(*r.prims, pj.prim_off, pj.nprims);
        pj.prims = pj.stroke_gpu ? r.dstroke : r.dprims;
        pj.pc_off = pc;
        pc += pj.nprims;
        pj.img = r.canvas->data;
        pj.W = r.canvas->width;
        pj.H = r.canvas->height;
        pj.row_off = recItems;  // recording items: one per row of the canvas
        recItems += pj.H;
        pj.ri_off = s.ri_base + (long long)(j - r.j0);
        pj.ri_stride = nrun;
        pj.status = kOk;
        dev.push_back(pj);
      }
      s.j1 = (int)dev.size();
      riTotal += s.H * nrun;
      items += s.H * ((s.W + slice - 1) / slice);
      maxH = std::max<long long>(maxH, s.H);
      sr.push_back(s);
      which.push_back(ri);
    }
    if (sr.empty()) return;
    const int nj = (int)dev.size();
    const int maxBands = setup_max_bands(maxH);
    ensure_arena(seg_need, list_need, (long long)nj * maxBands, pc, 1);
    if (prog_need == 0) prog_need = std::max<long long>(1 << 20, std::min<long long>(recItems * 3, 1LL << 27));
    dev_grow(g.prog, g.prog_cap, prog_need);
    dev_grow(g.rowidx, g.rowidx_cap, std::max<long long>(riTotal, 1));
    if (!g.cov8) {  // coverage-byte arena: up to 4 GB, at most an eighth of the free memory
      size_t fr = 0, tot = 0;
      CU(cudaMemGetInfo(&fr, &tot));
      long long cap = std::min<long long>(4LL << 30, (long long)(fr / 8));
      cap = std::max<long long>(cap, 1 << 20);
      CU(cudaMalloc(&g.cov8, (size_t)cap));
      g.cov8_cap = cap;
    }
    const long long recBlocks = std::max<long long>(
        1, std::min<long long>((recItems + scene_rec_warps() - 1) / scene_rec_warps(),
                               (long long)g.nsm * g.scene_ctas_per_sm[0]));
    const long long slots = recBlocks * scene_rec_warps();
    if (slots > g.wide_slots) {
      if (g.wide) cudaFree(g.wide);
      g.wide = nullptr;
      g.wide_slots = 0;
      CU(cudaMalloc(&g.wide, (size_t)slots * scene_wide_bytes()));
      g.wide_slots = slots;
    }
    const long long blocks = std::max<long long>(
        1, std::min<long long>((items + scene_warps() - 1) / scene_warps(), (long long)g.nsm * g.scene_ctas_per_sm[1]));
    Staged S = stage(dev, sr.data(), sizeof(SceneRun) * sr.size(), std::vector<Prim>());
    k_setup<<<nj, 256, setup_smem(maxBands), g.stream>>>(S.dj, S.A, maxBands); note_launch();
    CU(cudaGetLastError());
    CU(cudaMemsetAsync(g.rowidx, 0xff, sizeof(int) * (size_t)std::max<long long>(riTotal, 1), g.stream));
    launch_scene_rec((unsigned)recBlocks, g.stream, S.dj, reinterpret_cast<const SceneRun*>(S.extra), (int)sr.size(),
                     recItems, S.A, g.wide, g.wide_slots);
    note_launch();
    CU(cudaGetLastError());
    launch_scene((unsigned)blocks, g.stream, S.dj, reinterpret_cast<const SceneRun*>(S.extra), (int)sr.size(), items,
                 S.A, g.tbl, slice);
    note_launch();
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(g.h_up, g.d_up, S.jobsBytes + S.ctrBytes, cudaMemcpyDeviceToHost, g.stream));
    CU(cudaStreamSynchronize(g.stream));
    unsigned long long ctr[kNumCounters];
    memcpy(ctr, g.h_up + S.jobsBytes, sizeof ctr);
    note_stats(nj, pc, ctr);
    if (ctr[kCtrProgFull]) {  // nothing was drawn: rerun with room for every program
      prog_need = std::max<long long>(prog_need * 2, (long long)(ctr[kCtrProg] + ctr[kCtrProg] / 4));
      continue;
    }
    const PathJob* out = reinterpret_cast<const PathJob*>(g.h_up);
    bool grow = false;
    for (size_t k = 0; k < sr.size(); k++) {
      HostRun& r = runs[which[k]];
      size_t done = r.j1;
      for (int j = sr[k].j0; j < sr[k].j1; j++) {
        const int st = out[j].status;
        if (st == kOk || st == kNothing) continue;
        done = r.j0 + (size_t)(j - sr[k].j0);
        if (st == kErrArenaFull) grow = true;
        else r.status = st;
        break;
      }
      if (ctr[kCtrRowErr] != ~0ull && (int)ctr[kCtrRowErr] >= sr[k].j0 && (int)ctr[kCtrRowErr] < sr[k].j1)
        r.status = kErrRowTooComplex;
      r.j0 = r.status == kOk ? done : r.j1;
    }
    if (!grow) return;
    grow_needs(ctr, seg_need, list_need);
  }
  for (auto& r : runs)
    if (r.status == kOk && r.j0 < r.j1) r.status = kErrArenaFull;
}

PathJob make_job(pxg_image* img, uint32_t rgbx, int blend, const float* mat, float ps, int winding) {
  PathJob j;
  memset(&j, 0, sizeof j);
  j.winding = winding;
  j.ems = error_margin_sq(ps);
  j.identity = is_identity(mat) ? 1 : 0;
  j.mode = blend;
  j.rgbx = rgbx;
  memcpy(j.mat, mat, sizeof j.mat);
  if (img) {
    j.img = img->data;
    j.W = img->width;
    j.H = img->height;
  }
  return j;
}

const float kIdent[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};

void check_image(const pxg_image* img) {
  if (!img || !img->data) throw ApiError{"Invalid image handle"};
}
void check_blend(int b) {
  if (b < 0 || b >= kNumBlends) throw ApiError{"Invalid blend mode"};
}

// fillPath's paint handling (paths.nim:2100-2112): returns false when nothing draws.
bool paint_color(const float* color, float& opacity, int blend, uint32_t& rgbx) {
  opacity = opacity < 0 ? 0 : (opacity > 1 ? 1 : opacity);
  if (opacity == 0) return false;
  if (!(color[3] > 0 || blend == kOverwrite)) return false;
  float c[4] = {color[0], color[1], color[2], color[3] * opacity};
  rgbx = color_to_rgbx(c);
  return true;
}

// Host-only work (recording geometry): no device needed.
template <class F>
int guarded_host(F&& f) {
  try {
    f();
    return 0;
  } catch (const ApiError& e) {
    set_err(e.msg);
  } catch (const GeomError& e) {
    set_err(e.msg);
  } catch (const std::exception& e) {
    set_err(e.what());
  }
  return 1;
}

// Compute issued from here on waits for the asynchronous copies issued so far.
void copy_fence() {
  for (cudaEvent_t e : g.copies_pending) {
    CU(cudaStreamWaitEvent(g.stream, e, 0));
    g.ev_pool.push_back(e);
  }
  g.copies_pending.clear();
}
cudaEvent_t pooled_event() {
  cudaEvent_t e = nullptr;
  if (!g.ev_pool.empty()) {
    e = g.ev_pool.back();
    g.ev_pool.pop_back();
  } else {
    CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  return e;
}
// An asynchronous copy on stream cs of image im: after the compute issued
// before it and the image's previous copy; compute issued after it waits.
template <class Copy>
void async_copy(pxg_image* im, cudaStream_t cs, Copy&& copy) {
  if (!g.async_copies) {  // the first one: the compute stream's position now
    g.async_copies = true;
    CU(cudaEventRecord(g.compute_ev, g.stream));
  }
  CU(cudaStreamWaitEvent(cs, g.compute_ev, 0));
  if (im->compute_set) CU(cudaStreamWaitEvent(cs, im->compute_ev, 0));
  if (im->copy_ev)
    CU(cudaStreamWaitEvent(cs, im->copy_ev, 0));
  else
    CU(cudaEventCreateWithFlags(&im->copy_ev, cudaEventDisableTiming));
  copy();
  CU(cudaEventRecord(im->copy_ev, cs));
  im->copy_pending = true;
  cudaEvent_t e = pooled_event();
  CU(cudaEventRecord(e, cs));
  g.copies_pending.push_back(e);
  // calls that name their images never drain the list; keep it bounded (the
  // compute stream then waits for all of them: conservative, still correct)
  if (g.copies_pending.size() > 1024) copy_fence();
}

// Every entry point runs through guarded.  A compute call first waits for
// the asynchronous copies issued before it and afterwards records the compute
// stream's position for later copies; a copy call (COPY) does neither -- it
// waits for that recorded position, so it is not ordered after other copies.
template <bool COPY = false, class F>
int guarded(F&& f) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  try {
    ensure_init();
    if (!COPY && !g.copies_pending.empty()) copy_fence();
    f();
    if (!COPY && g.async_copies) CU(cudaEventRecord(g.compute_ev, g.stream));
    return 0;
  } catch (const ApiError& e) {
    set_err(e.msg);
  } catch (const GeomError& e) {
    set_err(e.msg);
  } catch (const std::exception& e) {
    set_err(e.what());
  }
  return 1;
}

// A compute call that names the images it reads and writes: it waits only for
// those images' asynchronous copies, so it can start while copies of other
// images are still running, and records an event on each of them, so later
// copies of those images wait for it and not for unrelated compute.  (The
// global position g.compute_ev moves only with calls that do not name their
// images.)
template <class F>
int guarded_images(std::initializer_list<const pxg_image*> ims, F&& f) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  try {
    ensure_init();
    for (const pxg_image* c : ims) {
      pxg_image* im = const_cast<pxg_image*>(c);
      if (im && im->copy_pending) {
        CU(cudaStreamWaitEvent(g.stream, im->copy_ev, 0));
        im->copy_pending = false;
      }
    }
    f();
    if (g.async_copies)  // later copies of these images wait for this call only
      for (const pxg_image* c : ims) {
        pxg_image* im = const_cast<pxg_image*>(c);
        if (!im) continue;
        if (!im->compute_ev) CU(cudaEventCreateWithFlags(&im->compute_ev, cudaEventDisableTiming));
        CU(cudaEventRecord(im->compute_ev, g.stream));
        im->compute_set = true;
      }
    return 0;
  } catch (const ApiError& e) {
    set_err(e.msg);
  } catch (const GeomError& e) {
    set_err(e.msg);
  } catch (const std::exception& e) {
    set_err(e.what());
  }
  return 1;
}

void run_single(pxg_image* img, std::vector<Prim>& prims, uint32_t rgbx, int blend,
                const float* mat, float ps, int winding) {
  std::vector<PathJob> jobs(1, make_job(img, rgbx, blend, mat, ps, winding));
  jobs[0].prim_off = 0;
  jobs[0].nprims = (int)prims.size();
  std::vector<int> st;
  Timed t(true);
  run_jobs(jobs, prims, st);
  t.done();
  if (st[0] != kOk) throw ApiError{status_message(st[0])};
}

// ---------------------------------------------------------------------------
// Serving engine
// ---------------------------------------------------------------------------
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Canvases come from the device's stream-ordered memory pool: allocation and
// release are ordered on the library's stream and never synchronise the
// device, and freed blocks stay in the pool for the next admissions.
void srv_pool_init() {
  static bool done = false;
  if (done) return;
  cudaMemPool_t pool;
  CU(cudaDeviceGetDefaultMemPool(&pool, g.dev));
  uint64_t keep = ~0ull;
  CU(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  done = true;
}

constexpr long long kStepPathRows = 8LL << 20;

void srv_release(pxg_server* sv, SrvJob* j) {
  if (j->canvas.data) cudaFreeAsync(j->canvas.data, g.stream);
  if (j->tmp) cudaFreeAsync(j->tmp, g.stream);
  j->canvas.data = nullptr;
  j->tmp = nullptr;
  sv->used -= j->bytes;
  j->bytes = 0;
}

// Device bytes a job holds while admitted: its canvas, and the blur's
// intermediate buffer when it is blurred.
long long srv_job_bytes(long long W, long long H, int64_t blur) {
  return W * H * 4 + (blur > 0 ? blur_scratch_bytes(W, H) : 0);
}

// Admits queued jobs in arrival order while their canvases fit the budget.
void srv_admit(pxg_server* sv) {
  while (!sv->queue.empty()) {
    SrvJob* j = sv->queue.front();
    const long long need = srv_job_bytes(j->W, j->H, j->blur);
    if (sv->used + need > sv->budget) break;
    sv->queue.pop_front();
    srv_pool_init();
    CU(cudaMallocAsync((void**)&j->canvas.data, (size_t)(j->W * j->H * 4), g.stream));
    j->canvas.width = j->W;
    j->canvas.height = j->H;
    j->canvas.owned = 1;
    if (j->blur > 0) CU(cudaMallocAsync((void**)&j->tmp, (size_t)blur_scratch_bytes(j->W, j->H), g.stream));
    CU(cudaMemsetAsync(j->canvas.data, 0, (size_t)(j->W * j->H * 4), g.stream));
    j->bytes = need;
    sv->used += need;
    sv->peak_used = std::max(sv->peak_used, sv->used);
    j->state = 1;
    j->t_admit = now_s();
    sv->active.push_back(j);
  }
  sv->peak_active = std::max<long long>(sv->peak_active, (long long)sv->active.size());
}

void srv_finish(pxg_server* sv, SrvJob* j, int status, const std::string& err) {
  j->status = status;
  j->err = err;
  j->state = status == kOk ? 2 : 3;
  j->t_done = now_s();
  sv->finished.push_back(j->id);
}

// One step: every active job's next chunk of paths in one setup + scene
// launch pair; MaskBlend paths run alone; finished jobs get their blur.
void srv_step(pxg_server* sv) {
  srv_admit(sv);
  if (sv->active.empty()) return;
  std::vector<HostRun> runs;
  std::vector<SrvJob*> owners;
  std::vector<std::vector<PathJob>*> jobvecs;
  long long budget = sv->paths_per_step;
  long long rowBudget = kStepPathRows;  // path-rows of the step: bounds its row programs
  for (SrvJob* j : sv->active) {
    if (budget <= 0 || rowBudget <= 0) break;
    const auto& pj = j->scene->jobs;
    if (j->next < pj.size() && pj[j->next].mode == kMask) {
      // a MaskBlend path: drawn alone
      PathJob one = pj[j->next];
      std::vector<Prim> sub(j->scene->prims.begin() + one.prim_off,
                            j->scene->prims.begin() + one.prim_off + one.nprims);
      one.prim_off = 0;
      one.img = j->canvas.data;
      one.W = j->W;
      one.H = j->H;
      std::vector<PathJob> v(1, one);
      std::vector<int> st;
      run_jobs(v, sub, st);
      if (st[0] != kOk) {
        srv_finish(sv, j, st[0], status_message(st[0]));
        continue;
      }
      j->next++;
      budget--;
      continue;
    }
    size_t e = j->next;
    const size_t lim = (size_t)std::max<long long>(
        1, std::min<long long>(std::min<long long>(sv->paths_per_job, budget), rowBudget / j->H));
    while (e < pj.size() && e - j->next < lim && pj[e].mode != kMask) e++;
    if (e == j->next) continue;
    rowBudget -= (long long)(e - j->next) * j->H;
    runs.push_back(HostRun{&j->canvas, const_cast<std::vector<PathJob>*>(&pj), &j->scene->prims,
                           scene_device_prims(j->scene), j->next, e, kOk, j->scene->dstroke});
    owners.push_back(j);
    budget -= (long long)(e - j->next);
  }
  if (!runs.empty()) {
    std::vector<size_t> ends;
    for (auto& r : runs) ends.push_back(r.j1);
    run_scene_runs(runs);
    for (size_t k = 0; k < runs.size(); k++) {
      SrvJob* j = owners[k];
      if (j->state != 1) continue;
      if (runs[k].status != kOk) srv_finish(sv, j, runs[k].status, status_message(runs[k].status));
      else j->next = ends[k];
    }
  }
  // jobs whose paths are all painted: blur, then done
  std::vector<SrvJob*> still;
  std::vector<SrvJob*> done;
  for (SrvJob* j : sv->active) {
    if (j->state != 1) {
      srv_release(sv, j);
      continue;
    }
    if (j->next >= j->scene->jobs.size()) {
      if (j->blur > 0) {
        if (blur_dispatch((uint32_t*)j->canvas.data, (uint32_t*)j->tmp, blur_scratch_bytes(j->W, j->H), j->W, j->H,
                          j->blur, 0u, true))
          std::swap(j->canvas.data, j->tmp);  // both the job's own; the old canvas is freed with tmp below
        CU(cudaGetLastError());
      }
      done.push_back(j);
    } else {
      still.push_back(j);
    }
  }
  if (!done.empty()) CU(cudaStreamSynchronize(g.stream));
  for (SrvJob* j : done) {
    srv_finish(sv, j, kOk, "");
    if (j->tmp) {
      cudaFreeAsync(j->tmp, g.stream);
      j->tmp = nullptr;
      const long long half = j->W * j->H * 4;
      sv->used -= half;
      j->bytes -= half;
    }
  }
  sv->active = still;
  sv->steps++;
}

// ---------------------------------------------------------------------------
// Autotuner: per operation and shape class, the fastest of a few launch
// configurations, found by timing each once the first time the class is
// seen.  Every configuration computes the same bytes; only speed differs.
// ---------------------------------------------------------------------------
enum TuneOp { kTuneMaskRows = 0, kTuneMaskDraw = 1 };
const RowsCfg kMaskRowsCands[] = {{0, 1}, {1, 1}, {1, 2}, {1, 4}};
constexpr int kNumMaskRowsCands = 4;

struct Tuner {
  bool on = true;
  std::map<std::pair<int, long long>, int> best;
  std::map<std::pair<int, long long>, std::vector<float>> ms;
};
Tuner g_tune;

int size_bucket(long long v) {  // 0: <=32, 1: <=64, ... 6: >1024
  int b = 0;
  long long lim = 32;
  while (b < 6 && v > lim) {
    lim *= 2;
    b++;
  }
  return b;
}
int count_bucket(long long n) {
  int b = 0;
  while (b < 20 && (1LL << b) < n) b++;
  return b;
}
long long mask_class(const pxg_masks* m) {
  long long side = 1;
  for (const PathJob& j : m->jobs) side = std::max<long long>(side, std::max<long long>(j.W, j.H));
  return size_bucket(side) * 32 + count_bucket((long long)m->jobs.size());
}

}  // namespace

struct GraphCacheHolder {
  GraphCache gc;
};
pxg_server::~pxg_server() {
  for (auto& kv : jobs) {
    SrvJob* j = kv.second;
    if (j->canvas.data) cudaFreeAsync(j->canvas.data, g.stream);
    if (j->tmp) cudaFreeAsync(j->tmp, g.stream);
    delete j;
  }
  if (g.ready) cudaStreamSynchronize(g.stream);
}
pxg_masks::~pxg_masks() {
  if (graph) {
    graph->gc.reset();
    delete graph;
  }
  if (dev) cudaFree(dev);
  if (dprims) cudaFree(dprims);
}

namespace {

const Prim* masks_device_prims(pxg_masks* m) {
  if (m->dirty) {
    dev_grow(m->dprims, m->dcap, std::max<long long>((long long)m->prims.size(), 1));
    if (!m->prims.empty())
      CU(cudaMemcpy(m->dprims, m->prims.data(), sizeof(Prim) * m->prims.size(), cudaMemcpyHostToDevice));
    m->dirty = false;
  }
  return m->dprims;
}

void render_masks(pxg_masks* m) {
  if (m->jobs.empty()) return;
  dev_grow(m->dev, m->dev_cap, std::max<long long>(m->bytes, 16));
  std::vector<PathJob> jobs = m->jobs;
  for (size_t i = 0; i < jobs.size(); i++) jobs[i].img = m->dev + m->offs[i];
  if (!m->graph) m->graph = new GraphCacheHolder();
  const std::pair<int, long long> key{kTuneMaskRows, mask_class(m)};
  auto it = g_tune.best.find(key);
  std::vector<int> st;
  if (g_tune.on && it == g_tune.best.end()) {
    std::vector<float> t(kNumMaskRowsCands, 0.0f);
    int best = 0;
    for (int c = 0; c < kNumMaskRowsCands; c++) {
      std::vector<PathJob> jc = jobs;
      RunOpts o;
      o.cfg = kMaskRowsCands[c];
      o.zero = m->dev;
      o.zero_bytes = m->bytes;
      o.rows_ms = &t[(size_t)c];
      o.dprims = masks_device_prims(m);
      run_jobs(jc, m->prims, st, o);
      if (t[(size_t)c] < t[(size_t)best]) best = c;
    }
    g_tune.best[key] = best;
    g_tune.ms[key] = t;
  } else {
    RunOpts o;
    o.cfg = kMaskRowsCands[it == g_tune.best.end() ? 1 : it->second];
    o.zero = m->dev;
    o.zero_bytes = m->bytes;
    o.graph = &m->graph->gc;
    o.dprims = masks_device_prims(m);
    run_jobs(jobs, m->prims, st, o);
  }
  for (size_t i = 0; i < st.size(); i++)
    if (st[i] != kOk) throw ApiError{status_message(st[i])};
  m->rendered = true;
}

void draw_masks(pxg_image* page, const pxg_masks* m, const int64_t* xy, int blend) {
  const int n = (int)m->jobs.size();
  if (n == 0) return;
  std::vector<MaskDraw> items((size_t)n);
  for (int i = 0; i < n; i++) {
    items[(size_t)i].off = m->offs[(size_t)i];
    items[(size_t)i].x = xy[2 * i];
    items[(size_t)i].y = xy[2 * i + 1];
    items[(size_t)i].w = (int)m->jobs[(size_t)i].W;
    items[(size_t)i].h = (int)m->jobs[(size_t)i].H;
  }
  // a pageable copy: the host vector may go away as soon as the call returns
  dev_grow(g.mdraw, g.mdraw_cap, (long long)n);
  CU(cudaMemcpyAsync(g.mdraw, items.data(), sizeof(MaskDraw) * (size_t)n, cudaMemcpyHostToDevice, g.stream));
  struct {
    const void* extra;
  } S{g.mdraw};
  const long long pxBytes = page->width * page->height * 4;
  const std::pair<int, long long> key{kTuneMaskDraw, size_bucket(std::max(page->width, page->height)) * 32 +
                                                        count_bucket(n)};
  auto it = g_tune.best.find(key);
  int tile = 2;
  if (g_tune.on && it == g_tune.best.end()) {
    // time every tile shape on a copy of the page, then draw with the fastest
    unsigned char* tmp = (unsigned char*)scratch(pxBytes);
    std::vector<float> t((size_t)draw_masks_tiles(), 0.0f);
    for (int c = 0; c < draw_masks_tiles(); c++) {
      CU(cudaMemcpyAsync(tmp, page->data, (size_t)pxBytes, cudaMemcpyDeviceToDevice, g.stream));
      CU(cudaEventRecord(g.evr0, g.stream));
      launch_draw_masks(c, (uint32_t*)tmp, page->width, page->height, S.extra, n, m->dev, blend, g.tbl, g.stream);
      CU(cudaGetLastError());
      CU(cudaEventRecord(g.evr1, g.stream));
      CU(cudaEventSynchronize(g.evr1));
      CU(cudaEventElapsedTime(&t[(size_t)c], g.evr0, g.evr1));
      if (t[(size_t)c] < t[(size_t)tile]) tile = c;
    }
    g_tune.best[key] = tile;
    g_tune.ms[key] = t;
  } else if (it != g_tune.best.end()) {
    tile = it->second;
  }
  launch_draw_masks(tile, (uint32_t*)page->data, page->width, page->height, S.extra, n, m->dev, blend, g.tbl,
                    g.stream);
  CU(cudaGetLastError());
}

}  // namespace

namespace pxg {
// Records an error for pxg_take_error() without allocating.
void record_error(const char* msg) { set_err(msg); }
}  // namespace pxg

extern "C" {

int pxg_check_error(void) { return t_has_err ? 1 : 0; }

const char* pxg_take_error(void) {
  snprintf(t_taken, sizeof t_taken, "%s", t_has_err ? t_err : "");
  t_err[0] = 0;
  t_has_err = false;
  return t_taken;
}

int pxg_init(int device) {
  return guarded([&] {
    if (g.ready && g.dev != device) throw ApiError{"pxg is already initialised on another device"};
    init_locked(device);
  });
}

int pxg_set_stream(void* s) {
  return guarded([&] { g.stream = s ? (cudaStream_t)s : g.own; });
}

int pxg_synchronize(void) {
  return guarded([&] {
    CU(cudaStreamSynchronize(g.stream));
    if (g.async_copies) {
      CU(cudaStreamSynchronize(g.h2d));
      CU(cudaStreamSynchronize(g.d2h));
    }
  });
}

float pxg_last_gpu_ms(void) { return g.last_ms; }

int pxg_set_blocking(int blocking) {
  return guarded([&] {
    if (blocking && !g.blocking && g.async_copies) {  // back to blocking: finish the asynchronous copies
      CU(cudaStreamSynchronize(g.h2d));
      CU(cudaStreamSynchronize(g.d2h));
    }
    g.blocking = blocking != 0;
  });
}

int64_t pxg_launch_count(void) { return (int64_t)launch_count(); }

pxg_image* pxg_new_image(int64_t width, int64_t height) {
  pxg_image* out = nullptr;
  guarded([&] {
    if (width <= 0 || height <= 0) throw ApiError{"Image width and height must be > 0"};
    pxg_image* im = new pxg_image{nullptr, width, height, 1};
    // room for a blur's padded intermediate too, so that the buffers a blur
    // swaps between an image and the scratch buffer keep serving both
    im->cap = blur_scratch_bytes(width, height);
    cudaError_t e = cudaMalloc((void**)&im->data, (size_t)im->cap);
    if (e != cudaSuccess) {
      delete im;
      throw ApiError{std::string("CUDA error: ") + cudaGetErrorString(e)};
    }
    e = cudaMemsetAsync(im->data, 0, (size_t)(width * height * 4), g.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.stream);
    if (e != cudaSuccess) {
      cudaFree(im->data);
      delete im;
      throw ApiError{std::string("CUDA error: ") + cudaGetErrorString(e)};
    }
    out = im;
  });
  return out;
}

pxg_image* pxg_image_wrap(void* ptr, int64_t width, int64_t height) {
  pxg_image* out = nullptr;
  guarded([&] {
    if (width <= 0 || height <= 0) throw ApiError{"Image width and height must be > 0"};
    if (!ptr || ((uintptr_t)ptr & 15)) throw ApiError{"Device pointer must be non-null and 16-byte aligned"};
    out = new pxg_image{(uint8_t*)ptr, width, height, 0};
  });
  return out;
}

void pxg_image_free(pxg_image* im) {
  if (!im) return;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (im->copy_ev) {  // a copy may still be in flight on the image's memory
    cudaEventSynchronize(im->copy_ev);
    cudaEventDestroy(im->copy_ev);
  }
  if (im->compute_ev) cudaEventDestroy(im->compute_ev);
  if (im->owned && im->data) cudaFree(im->data);
  delete im;
}

int64_t pxg_image_width(const pxg_image* im) { return im ? im->width : 0; }
int64_t pxg_image_height(const pxg_image* im) { return im ? im->height : 0; }
void* pxg_image_device_ptr(pxg_image* im) {
  if (!im) return nullptr;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  im->exported = true;
  return im->data;
}

int pxg_image_upload(pxg_image* im, const void* host, int64_t nbytes) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);  // the mode is read and used under the library's lock
  if (!g.blocking)
    return guarded<true>([&] {  // on the upload stream; the host buffer must stay as it is until pxg_synchronize
      check_image(im);
      if (nbytes != im->width * im->height * 4) throw ApiError{"Byte count does not match the image"};
      async_copy(im, g.h2d, [&] {
        CU(cudaMemcpyAsync(im->data, host, (size_t)nbytes, cudaMemcpyHostToDevice, g.h2d));
      });
    });
  return guarded([&] {
    check_image(im);
    if (nbytes != im->width * im->height * 4) throw ApiError{"Byte count does not match the image"};
    CU(cudaMemcpyAsync(im->data, host, (size_t)nbytes, cudaMemcpyHostToDevice, g.stream));
    CU(cudaStreamSynchronize(g.stream));
  });
}

int pxg_image_download(const pxg_image* im, void* host, int64_t nbytes) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);  // the mode is read and used under the library's lock
  if (!g.blocking)
    return guarded<true>([&] {  // on the download stream; the host buffer holds the image after pxg_synchronize
      check_image(im);
      if (nbytes != im->width * im->height * 4) throw ApiError{"Byte count does not match the image"};
      pxg_image* m = const_cast<pxg_image*>(im);
      async_copy(m, g.d2h, [&] {
        CU(cudaMemcpyAsync(host, im->data, (size_t)nbytes, cudaMemcpyDeviceToHost, g.d2h));
      });
    });
  return guarded([&] {
    check_image(im);
    if (nbytes != im->width * im->height * 4) throw ApiError{"Byte count does not match the image"};
    CU(cudaMemcpyAsync(host, im->data, (size_t)nbytes, cudaMemcpyDeviceToHost, g.stream));
    CU(cudaStreamSynchronize(g.stream));
  });
}

int pxg_image_fill(pxg_image* im, const float* color) {
  return guarded_images({im}, [&] {
    check_image(im);
    Timed t;
    launch_fill((uint32_t*)im->data, im->width * im->height, color_to_rgbx(color), g.nsm, g.stream);
    CU(cudaGetLastError());
    t.done();
  });
}

int pxg_image_fill_path(pxg_image* im, const float* cmds, int64_t n, const float* color,
                        float opacity, int blend, const float* transform, int winding) {
  return guarded([&] {
    check_image(im);
    check_blend(blend);
    if (winding != 0 && winding != 1) throw ApiError{"Invalid winding rule"};
    if (n < 0 || (n > 0 && !cmds)) throw ApiError{"Invalid path commands"};
    validate_commands(cmds, n);
    uint32_t rgbx;
    if (!paint_color(color, opacity, blend, rgbx)) return;
    const float* mat = transform ? transform : kIdent;
    float ps = pixel_scale(mat);
    std::vector<Prim> prims;
    build_fill_prims(cmds, n, ps, prims);
    run_single(im, prims, rgbx, blend, mat, ps, winding);
  });
}

int pxg_image_stroke_path(pxg_image* im, const float* cmds, int64_t n, const float* color,
                          float opacity, int blend, const float* transform, float width, int cap,
                          int join, float miterLimit, const float* dashes, int64_t nd) {
  return guarded([&] {
    check_image(im);
    check_blend(blend);
    if (n < 0 || (n > 0 && !cmds)) throw ApiError{"Invalid path commands"};
    validate_commands(cmds, n);
    uint32_t rgbx;
    if (!paint_color(color, opacity, blend, rgbx)) return;
    const float* mat = transform ? transform : kIdent;
    float ps = pixel_scale(mat);
    StrokeGeom sg;
    if (g.stroke_gpu && build_stroke_geom(cmds, n, ps, width, cap, join, miterLimit, nd, sg) && sg.nprims > 0) {
      if (sg.nprims > INT32_MAX) throw ApiError{"Path too complex"};
      Timed t(true);
      dev_grow(g.sk_prims, g.sk_prims_cap, sg.nprims);
      outline_strokes(sg, g.sk_prims);
      std::vector<PathJob> jobs(1, make_job(im, rgbx, blend, mat, ps, 0));
      jobs[0].prim_off = 0;
      jobs[0].nprims = (int)sg.nprims;
      jobs[0].group = group_for(sg.ncurves);
      RunOpts opts;
      opts.dprims = g.sk_prims;
      opts.ndprims = sg.nprims;
      std::vector<int> st;
      run_jobs(jobs, std::vector<Prim>(), st, opts);
      t.done();
      if (st[0] != kOk) throw ApiError{status_message(st[0])};
      return;
    }
    std::vector<Prim> prims;
    build_stroke_prims(cmds, n, ps, width, cap, join, miterLimit, dashes, nd, prims);
    run_single(im, prims, rgbx, blend, mat, ps, 0);
  });
}

int pxg_fill_paths_batch(pxg_image* const* images, int64_t nj, const float* cmds,
                         const int64_t* offs, const float* colors, const float* opacities,
                         const int32_t* blends, const float* transforms, const int32_t* windings,
                         int32_t* status) {
  return guarded([&] {
    std::vector<Prim> prims, tmp;
    std::vector<PathJob> jobs;
    std::vector<int64_t> index;  // job -> caller index
    for (int64_t j = 0; j < nj; j++) {
      if (status) status[j] = 0;
      pxg_image* im = images[j];
      check_image(im);
      check_blend(blends[j]);
      float op = opacities ? opacities[j] : 1.0f;
      uint32_t rgbx;
      const float* col = colors + 4 * j;
      const float* mat = transforms ? transforms + 9 * j : kIdent;
      const float* c = cmds + offs[j];
      int64_t n = offs[j + 1] - offs[j];
      try {
        validate_commands(c, n);
        if (!paint_color(col, op, blends[j], rgbx)) continue;
        float ps = pixel_scale(mat);
        build_fill_prims(c, n, ps, tmp);
        PathJob pj = make_job(im, rgbx, blends[j], mat, ps, windings ? windings[j] : 0);
        pj.prim_off = (long long)prims.size();
        pj.nprims = (int)tmp.size();
        prims.insert(prims.end(), tmp.begin(), tmp.end());
        jobs.push_back(pj);
        index.push_back(j);
      } catch (const GeomError&) {
        if (status) status[j] = kErrCubic;
      }
    }
    std::vector<int> st;
    Timed t(true);
    if (!jobs.empty()) run_jobs(jobs, prims, st);
    t.done();
    int bad = 0;
    for (size_t k = 0; k < jobs.size(); k++) {
      if (status) status[index[k]] = st[k];
      if (st[k] != kOk && !bad) bad = st[k];
    }
    if (bad) throw ApiError{status_message(bad)};
  });
}

int pxg_last_fill_stats(int64_t* out6) {
  if (!out6) {
    set_err("Invalid output pointer");
    return 1;
  }
  for (int i = 0; i < 6; i++) out6[i] = g.stats[i];
  return 0;
}

pxg_scene* pxg_scene_new(void) {
  try {
    return new pxg_scene();
  } catch (...) {
    set_err("Out of host memory");
    return nullptr;
  }
}

void pxg_scene_free(pxg_scene* sc) { delete sc; }

int pxg_scene_clear(pxg_scene* sc) {
  if (!sc) {
    set_err("Invalid scene handle");
    return 1;
  }
  sc->prims.clear();
  sc->jobs.clear();
  sc->sk = StrokeGeom();
  sc->dirty = true;
  return 0;
}

int64_t pxg_scene_len(const pxg_scene* sc) { return sc ? (int64_t)sc->jobs.size() : 0; }

int pxg_scene_fill_path(pxg_scene* sc, const float* cmds, int64_t n, const float* color, float opacity,
                        int blend, const float* transform, int winding) {
  return guarded_host([&] {
    if (!sc) throw ApiError{"Invalid scene handle"};
    check_blend(blend);
    if (winding != 0 && winding != 1) throw ApiError{"Invalid winding rule"};
    if (n < 0 || (n > 0 && !cmds)) throw ApiError{"Invalid path commands"};
    validate_commands(cmds, n);
    uint32_t rgbx;
    if (!paint_color(color, opacity, blend, rgbx)) return;
    const float* mat = transform ? transform : kIdent;
    float ps = pixel_scale(mat);
    thread_local std::vector<Prim> prims;  // keeps its capacity between recordings
    build_fill_prims(cmds, n, ps, prims);
    PathJob j = make_job(nullptr, rgbx, blend, mat, ps, winding);
    j.prim_off = (long long)sc->prims.size();
    j.nprims = (int)prims.size();
    j.group = curve_group(prims, 0, j.nprims);
    sc->prims.insert(sc->prims.end(), prims.begin(), prims.end());
    sc->jobs.push_back(j);
    sc->dirty = true;
  });
}

int pxg_scene_stroke_path(pxg_scene* sc, const float* cmds, int64_t n, const float* color, float opacity,
                          int blend, const float* transform, float width, int cap, int join,
                          float miterLimit, const float* dashes, int64_t nd) {
  return guarded_host([&] {
    if (!sc) throw ApiError{"Invalid scene handle"};
    check_blend(blend);
    if (n < 0 || (n > 0 && !cmds)) throw ApiError{"Invalid path commands"};
    validate_commands(cmds, n);
    uint32_t rgbx;
    if (!paint_color(color, opacity, blend, rgbx)) return;
    const float* mat = transform ? transform : kIdent;
    float ps = pixel_scale(mat);
    PathJob j = make_job(nullptr, rgbx, blend, mat, ps, 0);
    thread_local StrokeGeom sg;
    if (g.stroke_gpu && blend != kMask &&
        build_stroke_geom(cmds, n, ps, width, cap, join, miterLimit, nd, sg) && sg.nprims > 0) {
      // the outline is built on the GPU when the scene is next uploaded
      if (sg.nprims > INT32_MAX) throw ApiError{"Path too complex"};
      j.stroke_gpu = 1;
      j.nprims = (int)sg.nprims;
      j.group = group_for(sg.ncurves);
      j.prim_off = append_stroke(sc->sk, sg);
      sc->jobs.push_back(j);
      sc->dirty = true;
      return;
    }
    thread_local std::vector<Prim> prims;  // keeps its capacity between recordings
    build_stroke_prims(cmds, n, ps, width, cap, join, miterLimit, dashes, nd, prims);
    j.prim_off = (long long)sc->prims.size();
    j.nprims = (int)prims.size();
    j.group = curve_group(prims, 0, j.nprims);
    sc->prims.insert(sc->prims.end(), prims.begin(), prims.end());
    sc->jobs.push_back(j);
    sc->dirty = true;
  });
}

// n recordings at once: each path's geometry (the command walk, arcs, stroke
// outlines) is built on a pool of host threads, independently, and the paths
// are appended in submission order -- the scene n calls of
// pxg_scene_fill_path / pxg_scene_stroke_path would build.
int pxg_scene_record_batch(pxg_scene* sc, int64_t n, const int32_t* kinds, const float* cmds, const int64_t* offs,
                           const float* colors, const float* opacities, const int32_t* blends,
                           const float* transforms, const int32_t* windings, const float* widths,
                           const int32_t* caps, const int32_t* joins, const float* miters, int32_t* status,
                           int threads) {
  return guarded_host([&] {
    if (!sc) throw ApiError{"Invalid scene handle"};
    if (n < 0 || (n > 0 && (!kinds || !cmds || !offs || !colors || !opacities || !blends)))
      throw ApiError{"Invalid batch"};
    struct Rec {
      std::vector<Prim> prims;
      StrokeGeom sg;  // a stroke outlined on the GPU (job.stroke_gpu)
      PathJob job;
      int state = 0;  // 0 nothing to draw, 1 recorded, 2 failed
      std::string err;
    };
    const bool strokeGpu = g.stroke_gpu;
    std::vector<Rec> rec((size_t)n);
    auto build = [&](int64_t i) {
      Rec& r = rec[(size_t)i];
      try {
        const int blend = blends[i];
        check_blend(blend);
        const int64_t a = offs[i], b = offs[i + 1];
        if (a < 0 || b < a) throw ApiError{"Invalid path commands"};
        validate_commands(cmds + a, b - a);
        uint32_t rgbx;
        float op = opacities[i];
        if (!paint_color(colors + 4 * i, op, blend, rgbx)) return;
        const float* mat = transforms ? transforms + 9 * i : kIdent;
        const float ps = pixel_scale(mat);
        int winding = 0;
        if (kinds[i] == 0) {
          winding = windings ? windings[i] : 0;
          if (winding != 0 && winding != 1) throw ApiError{"Invalid winding rule"};
          build_fill_prims(cmds + a, b - a, ps, r.prims);
        } else {
          if (!widths || !caps || !joins || !miters) throw ApiError{"Invalid batch"};
          if (strokeGpu && blend != kMask &&
              build_stroke_geom(cmds + a, b - a, ps, widths[i], caps[i], joins[i], miters[i], 0, r.sg) &&
              r.sg.nprims > 0) {
            if (r.sg.nprims > INT32_MAX) throw ApiError{"Path too complex"};
            r.job = make_job(nullptr, rgbx, blend, mat, ps, 0);
            r.job.stroke_gpu = 1;
            r.state = 1;
            return;
          }
          r.sg.shapes.clear();
          build_stroke_prims(cmds + a, b - a, ps, widths[i], caps[i], joins[i], miters[i], nullptr, 0, r.prims);
        }
        r.job = make_job(nullptr, rgbx, blend, mat, ps, winding);
        r.state = 1;
      } catch (const ApiError& e) {
        r.state = 2;
        r.err = e.msg;
      } catch (const GeomError& e) {
        r.state = 2;
        r.err = e.msg;
      } catch (const std::exception& e) {
        r.state = 2;
        r.err = e.what();
      }
    };
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    nt = std::max(1, std::min<int>(nt, (int)std::min<int64_t>(n / 4 + 1, 256)));
    std::atomic<int64_t> next{0};
    auto worker = [&] {
      for (int64_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) build(i);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    size_t total = sc->prims.size();
    for (const Rec& r : rec) total += r.state == 1 ? r.prims.size() : 0;
    sc->prims.reserve(total);  // one allocation: no regrowth copies of the scene's primitives
    sc->jobs.reserve(sc->jobs.size() + (size_t)n);
    std::string firstErr;
    for (int64_t i = 0; i < n; i++) {  // append in submission order
      Rec& r = rec[(size_t)i];
      if (status) status[i] = r.state == 2 ? 1 : 0;
      if (r.state == 2 && firstErr.empty()) firstErr = r.err;
      if (r.state != 1) continue;
      if (r.job.stroke_gpu) {
        r.job.nprims = (int)r.sg.nprims;
        r.job.group = group_for(r.sg.ncurves);
        r.job.prim_off = append_stroke(sc->sk, r.sg);
      } else {
        r.job.prim_off = (long long)sc->prims.size();
        r.job.nprims = (int)r.prims.size();
        r.job.group = curve_group(r.prims, 0, r.job.nprims);
        sc->prims.insert(sc->prims.end(), r.prims.begin(), r.prims.end());
      }
      sc->jobs.push_back(r.job);
      sc->dirty = true;
    }
    if (!firstErr.empty()) set_err(firstErr.c_str());  // reported, not raised: the other paths are recorded
  });
}

int pxg_image_draw_scene(pxg_image* im, const pxg_scene* sc) {
  return guarded([&] {
    check_image(im);
    if (!sc) throw ApiError{"Invalid scene handle"};
    std::vector<PathJob> jobs = sc->jobs;
    Timed t(true);
    const Prim* dp = scene_device_prims(sc);
    size_t i = 0;
    while (i < jobs.size()) {
      if (jobs[i].mode == kMask) {  // its clears cover rows outside its own: draw it alone
        std::vector<Prim> sub(sc->prims.begin() + jobs[i].prim_off,
                              sc->prims.begin() + jobs[i].prim_off + jobs[i].nprims);
        PathJob j = jobs[i];
        j.img = im->data;
        j.W = im->width;
        j.H = im->height;
        j.prim_off = 0;
        std::vector<PathJob> one(1, j);
        std::vector<int> st;
        run_jobs(one, sub, st);
        if (st[0] != kOk) throw ApiError{status_message(st[0])};
        i++;
        continue;
      }
      size_t e = i;
      while (e < jobs.size() && jobs[e].mode != kMask) e++;
      std::vector<HostRun> runs(1);
      runs[0] = HostRun{im, &jobs, &sc->prims, dp, i, e, kOk, sc->dstroke};
      run_scene_runs(runs);
      if (runs[0].status != kOk) throw ApiError{status_message(runs[0].status)};
      i = e;
    }
    t.done();
  });
}

pxg_masks* pxg_masks_new(void) {
  try {
    return new pxg_masks();
  } catch (...) {
    set_err("Out of host memory");
    return nullptr;
  }
}

void pxg_masks_free(pxg_masks* m) {
  if (!m) return;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  delete m;
}

int64_t pxg_masks_len(const pxg_masks* m) { return m ? (int64_t)m->jobs.size() : 0; }

int pxg_masks_add_path(pxg_masks* m, const float* cmds, int64_t n, int64_t width, int64_t height,
                       const float* transform, int winding) {
  return guarded_host([&] {
    if (!m) throw ApiError{"Invalid mask batch handle"};
    if (width <= 0 || height <= 0) throw ApiError{"Image width and height must be > 0"};
    if (width > (1 << 20) || height > (1 << 20)) throw ApiError{"Mask too large"};
    if (winding != 0 && winding != 1) throw ApiError{"Invalid winding rule"};
    if (n < 0 || (n > 0 && !cmds)) throw ApiError{"Invalid path commands"};
    validate_commands(cmds, n);
    const float* mat = transform ? transform : kIdent;
    float ps = pixel_scale(mat);
    std::vector<Prim> prims;
    build_fill_prims(cmds, n, ps, prims);
    static const float white[4] = {1, 1, 1, 1};
    PathJob j = make_job(nullptr, color_to_rgbx(white), kNormal, mat, ps, winding);
    j.a8 = 1;
    j.W = width;
    j.H = height;
    j.prim_off = (long long)m->prims.size();
    j.nprims = (int)prims.size();
    j.group = curve_group(prims, 0, j.nprims);
    m->prims.insert(m->prims.end(), prims.begin(), prims.end());
    m->jobs.push_back(j);
    m->dirty = true;
    m->offs.push_back(m->bytes);
    m->bytes += (width * height + 15) / 16 * 16;
    m->rendered = false;
  });
}

// n glyphs at once, as n calls of pxg_masks_add_path would add them: the
// geometry is built on host threads and the masks are appended in order.
// All or nothing: if any path fails, none is added and the first failure is
// raised (a skipped glyph would shift the masks' indices).
int pxg_masks_add_paths(pxg_masks* m, int64_t n, const float* cmds, const int64_t* offs, const int64_t* widths,
                        const int64_t* heights, const float* transforms, const int32_t* windings, int threads) {
  return guarded_host([&] {
    if (!m) throw ApiError{"Invalid mask batch handle"};
    if (n < 0 || (n > 0 && (!cmds || !offs || !widths || !heights))) throw ApiError{"Invalid batch"};
    struct Rec {
      std::vector<Prim> prims;
      PathJob job;
      std::string err;
    };
    std::vector<Rec> rec((size_t)n);
    std::atomic<int> failed{0};
    auto build = [&](int64_t i) {
      Rec& r = rec[(size_t)i];
      try {
        const int64_t w = widths[i], h = heights[i];
        if (w <= 0 || h <= 0) throw ApiError{"Image width and height must be > 0"};
        if (w > (1 << 20) || h > (1 << 20)) throw ApiError{"Mask too large"};
        const int winding = windings ? windings[i] : 0;
        if (winding != 0 && winding != 1) throw ApiError{"Invalid winding rule"};
        const int64_t a = offs[i], b = offs[i + 1];
        if (a < 0 || b < a) throw ApiError{"Invalid path commands"};
        validate_commands(cmds + a, b - a);
        const float* mat = transforms ? transforms + 9 * i : kIdent;
        const float ps = pixel_scale(mat);
        build_fill_prims(cmds + a, b - a, ps, r.prims);
        static const float white[4] = {1, 1, 1, 1};
        r.job = make_job(nullptr, color_to_rgbx(white), kNormal, mat, ps, winding);
        r.job.a8 = 1;
        r.job.W = w;
        r.job.H = h;
      } catch (const ApiError& e) {
        r.err = e.msg;
        failed = 1;
      } catch (const GeomError& e) {
        r.err = e.msg;
        failed = 1;
      } catch (const std::exception& e) {
        r.err = e.what();
        failed = 1;
      }
    };
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    nt = std::max(1, std::min<int>(nt, (int)std::min<int64_t>(n / 16 + 1, 256)));
    std::atomic<int64_t> next{0};
    auto worker = [&] {
      for (int64_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) build(i);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    if (failed)
      for (const Rec& r : rec)
        if (!r.err.empty()) throw ApiError{r.err};
    size_t total = m->prims.size();
    for (const Rec& r : rec) total += r.prims.size();
    m->prims.reserve(total);
    for (int64_t i = 0; i < n; i++) {
      Rec& r = rec[(size_t)i];
      r.job.prim_off = (long long)m->prims.size();
      r.job.nprims = (int)r.prims.size();
      r.job.group = curve_group(r.prims, 0, r.job.nprims);
      m->prims.insert(m->prims.end(), r.prims.begin(), r.prims.end());
      m->jobs.push_back(r.job);
      m->offs.push_back(m->bytes);
      m->bytes += (r.job.W * r.job.H + 15) / 16 * 16;
    }
    if (n > 0) {
      m->dirty = true;
      m->rendered = false;
    }
  });
}

int pxg_masks_render(pxg_masks* m) {
  return guarded([&] {
    if (!m) throw ApiError{"Invalid mask batch handle"};
    Timed t(true);
    render_masks(m);
    t.done();
  });
}

int pxg_masks_render_config(pxg_masks* m, int variant, int rows_per_item) {
  return guarded([&] {
    if (!m) throw ApiError{"Invalid mask batch handle"};
    if (variant < 0 || variant > 1 || rows_per_item < 1 || rows_per_item > 64) throw ApiError{"Invalid configuration"};
    if (m->jobs.empty()) return;
    dev_grow(m->dev, m->dev_cap, std::max<long long>(m->bytes, 16));
    std::vector<PathJob> jobs = m->jobs;
    for (size_t i = 0; i < jobs.size(); i++) jobs[i].img = m->dev + m->offs[i];
    RunOpts o;
    o.cfg.variant = variant;
    o.cfg.rpi = rows_per_item;
    o.zero = m->dev;
    o.zero_bytes = m->bytes;
    o.dprims = masks_device_prims(m);
    std::vector<int> st;
    Timed t(true);
    run_jobs(jobs, m->prims, st, o);
    t.done();
    for (size_t i = 0; i < st.size(); i++)
      if (st[i] != kOk) throw ApiError{status_message(st[i])};
    m->rendered = true;
  });
}

int pxg_masks_download(const pxg_masks* m, int64_t i, void* out, int64_t nbytes) {
  return guarded([&] {
    if (!m) throw ApiError{"Invalid mask batch handle"};
    if (i < 0 || i >= (int64_t)m->jobs.size()) throw ApiError{"Mask index out of range"};
    if (!m->rendered) throw ApiError{"Masks not rendered"};
    const int64_t need = m->jobs[(size_t)i].W * m->jobs[(size_t)i].H;
    if (!out || nbytes < need) throw ApiError{"Output buffer too small"};
    CU(cudaStreamSynchronize(g.stream));
    CU(cudaMemcpy(out, m->dev + m->offs[(size_t)i], (size_t)need, cudaMemcpyDeviceToHost));
  });
}

const void* pxg_masks_device_ptr(const pxg_masks* m, int64_t i) {
  if (!m || i < 0 || i >= (int64_t)m->jobs.size() || !m->dev) return nullptr;
  return m->dev + m->offs[(size_t)i];
}

int pxg_image_draw_masks(pxg_image* page, const pxg_masks* m, const int64_t* xy, int blend) {
  return guarded([&] {
    check_image(page);
    if (!m) throw ApiError{"Invalid mask batch handle"};
    check_blend(blend);
    if (blend == kMask) throw ApiError{"MaskBlend is not supported for mask batches"};
    if (!m->rendered && !m->jobs.empty()) throw ApiError{"Masks not rendered"};
    if (!xy && !m->jobs.empty()) throw ApiError{"Invalid positions"};
    Timed t;
    draw_masks(page, m, xy, blend);
    t.done();
  });
}

pxg_server* pxg_server_new(int64_t budget_bytes, int64_t paths_per_job, int64_t paths_per_step) {
  try {
    if (budget_bytes <= 0 || paths_per_job <= 0 || paths_per_step <= 0) {
      set_err("Invalid server limits");
      return nullptr;
    }
    pxg_server* sv = new pxg_server();
    sv->budget = budget_bytes;
    sv->paths_per_job = paths_per_job;
    sv->paths_per_step = paths_per_step;
    return sv;
  } catch (...) {
    set_err("Out of host memory");
    return nullptr;
  }
}

void pxg_server_free(pxg_server* sv) {
  if (!sv) return;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (g.ready) cudaStreamSynchronize(g.stream);
  delete sv;
}

int64_t pxg_server_submit(pxg_server* sv, const pxg_scene* scene, int64_t width, int64_t height,
                          float blur_radius) {
  int64_t id = 0;
  int rc = guarded([&] {
    if (!sv || !scene) throw ApiError{"Invalid server or scene handle"};
    if (width <= 0 || height <= 0) throw ApiError{"Image width and height must be > 0"};
    const int64_t r = nim_round_int(blur_radius);
    if (r < 0) throw ApiError{"Cannot apply negative blur"};
    if (r > (1 << 20)) throw ApiError{"Blur radius too large"};
    const long long need = srv_job_bytes(width, height, r);
    if (need > sv->budget) throw ApiError{"Job larger than the server's memory budget"};
    SrvJob* j = new SrvJob();
    j->id = sv->next_id++;
    j->scene = scene;
    j->W = width;
    j->H = height;
    j->blur = r;
    j->state = 0;
    j->status = kOk;
    j->next = 0;
    j->bytes = 0;
    j->canvas = pxg_image{nullptr, 0, 0, 0};
    j->tmp = nullptr;
    j->t_submit = now_s();
    j->t_admit = j->t_done = 0;
    sv->jobs[j->id] = j;
    sv->queue.push_back(j);
    id = j->id;
  });
  return rc == 0 ? id : 0;
}

int pxg_server_step(pxg_server* sv) {
  return guarded([&] {
    if (!sv) throw ApiError{"Invalid server handle"};
    srv_step(sv);
  });
}

int64_t pxg_server_pending(const pxg_server* sv) {
  return sv ? (int64_t)(sv->queue.size() + sv->active.size()) : 0;
}

int64_t pxg_server_poll(pxg_server* sv, int64_t* ids, int64_t cap) {
  if (!sv) return 0;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  const int64_t n = std::min<int64_t>(cap, (int64_t)sv->finished.size());
  for (int64_t i = 0; i < n; i++) ids[i] = sv->finished[(size_t)i];
  sv->finished.erase(sv->finished.begin(), sv->finished.begin() + n);
  return n;
}

int pxg_server_take(pxg_server* sv, int64_t id, void* out, int64_t nbytes, double* times3) {
  return guarded([&] {
    if (!sv) throw ApiError{"Invalid server handle"};
    auto it = sv->jobs.find(id);
    if (it == sv->jobs.end()) throw ApiError{"Unknown job"};
    SrvJob* j = it->second;
    if (j->state < 2) throw ApiError{"Job not finished"};
    if (times3) {
      times3[0] = j->t_submit;
      times3[1] = j->t_admit;
      times3[2] = j->t_done;
    }
    std::string err = j->err;
    const int state = j->state;
    if (state == 2 && out) {
      if (nbytes < j->W * j->H * 4) throw ApiError{"Output buffer too small"};
      CU(cudaMemcpyAsync(out, j->canvas.data, (size_t)(j->W * j->H * 4), cudaMemcpyDeviceToHost, g.stream));
      CU(cudaStreamSynchronize(g.stream));
    }
    srv_release(sv, j);
    sv->jobs.erase(it);
    delete j;
    if (state == 3) throw ApiError{err};
  });
}

int pxg_server_stats(const pxg_server* sv, int64_t* out6) {
  if (!sv || !out6) {
    set_err("Invalid server handle");
    return 1;
  }
  out6[0] = sv->steps;
  out6[1] = sv->used;
  out6[2] = sv->peak_used;
  out6[3] = sv->peak_active;
  out6[4] = (int64_t)sv->queue.size();
  out6[5] = (int64_t)sv->active.size();
  return 0;
}

int pxg_scene_config(int slice_width, int64_t coverage_bytes) {
  return guarded([&] {
    if (slice_width != 0 && (slice_width < 32 || slice_width > (1 << 20)))
      throw ApiError{"Invalid scene configuration"};
    g.scene_slice = slice_width;
    if (coverage_bytes >= 0) {  // a new coverage-byte arena (0: spans only)
      CU(cudaStreamSynchronize(g.stream));
      if (g.cov8) cudaFree(g.cov8);
      g.cov8 = nullptr;
      g.cov8_cap = 0;
      CU(cudaMalloc(&g.cov8, (size_t)std::max<int64_t>(coverage_bytes, 16)));
      g.cov8_cap = coverage_bytes;
    }
  });
}

int pxg_stroke_config(int gpu_outline) {
  return guarded([&] {
    if (gpu_outline != 0 && gpu_outline != 1) throw ApiError{"Invalid stroke configuration"};
    g.stroke_gpu = gpu_outline != 0;
  });
}

int64_t pxg_stroke_fixups(void) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  return g.sk_fixups;
}

int pxg_blur_config(int use_tensor_cores) {
  return guarded([&] {
    if (use_tensor_cores < 0 || use_tensor_cores > 3) throw ApiError{"Invalid blur configuration"};
    g.blur_tensor = use_tensor_cores;
  });
}

int pxg_last_blur_kernel(void) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  return g.last_blur;
}

int pxg_ring_trace(int enable, int64_t* out, int64_t n) {
  return guarded([&] {
    CU(cudaDeviceSynchronize());
    if (ring_trace(enable, reinterpret_cast<long long*>(out), n) != 0) throw ApiError{"Ring blur trace unavailable"};
  });
}

int pxg_autotune(int enable) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  g_tune.on = enable != 0;
  return 0;
}

int64_t pxg_autotune_report(char* buf, int64_t cap) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  std::string r;
  for (auto& kv : g_tune.best) {
    char line[256];
    const int op = kv.first.first;
    const long long cls = kv.first.second;
    int c = kv.second;
    if (op == kTuneMaskRows)
      snprintf(line, sizeof line, "mask_rows class(side<=%d,count<=%lld): variant=%d rows_per_item=%d",
               32 << (int)(cls / 32), 1LL << (cls % 32), kMaskRowsCands[c].variant, kMaskRowsCands[c].rpi);
    else
      snprintf(line, sizeof line, "mask_draw class(side<=%d,count<=%lld): tile=%s", 32 << (int)(cls / 32),
               1LL << (cls % 32), c == 0 ? "32x32" : (c == 1 ? "64x32" : "64x64"));
    r += line;
    auto t = g_tune.ms.find(kv.first);
    if (t != g_tune.ms.end()) {
      r += " ms=[";
      for (size_t k = 0; k < t->second.size(); k++) {
        char v[32];
        snprintf(v, sizeof v, "%s%.4f", k ? "," : "", t->second[k]);
        r += v;
      }
      r += "]";
    }
    r += "\n";
  }
  if (buf && cap > 0) snprintf(buf, (size_t)cap, "%s", r.c_str());
  return (int64_t)r.size();
}

int pxg_image_draw(pxg_image* a, const pxg_image* b, int64_t tx, int64_t ty, int blend) {
  return guarded_images({a, b}, [&] {
    check_image(a);
    check_image(b);
    check_blend(blend);
    Timed t;
    launch_draw((uint32_t*)a->data, (const uint32_t*)b->data, a->width, a->height, b->width,
                b->height, tx, ty, blend, g.tbl, g.nsm, g.stream);
    CU(cudaGetLastError());
    t.done();
  });
}


}  // extern "C"

// ---------------------------------------------------------------------------
// draw with a Mat3 (images.nim:636-678).  The host does the reference's float32
// geometry (inverse, movement vectors, the minify/magnify decisions, the
// perimeter and row range of drawSmooth) in the same operations and order;
// the device resamples.  vmath's Mat3 is column-major: m[c * 3 + r], the
// translation in m[6], m[7].
// ---------------------------------------------------------------------------
namespace {
struct M3 {
  float m[9];
};
struct V {
  float x, y;
};
inline V m3v(const M3& M, float x, float y) {  // Mat3 * Vec2
  return V{M.m[0] * x + M.m[3] * y + M.m[6], M.m[1] * x + M.m[4] * y + M.m[7]};
}
inline V vsub(V a, V b) { return V{a.x - b.x, a.y - b.y}; }
inline float vlen(V v) { return sqrtf(v.x * v.x + v.y * v.y); }
inline float fnmax(float x, float y) { return y <= x ? x : y; }
inline float frac_abs(float v) {  // vmath fractional
  const float a = fabsf(v);
  return a - floorf(a);
}
inline int64_t h_nim_int(float f) {
  if (!(f >= -9223372036854775808.0f && f < 9223372036854775808.0f)) return INT64_MIN;
  return (int64_t)f;
}
inline int32_t h_nim_i32(float f) {
  if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
  return (int32_t)f;
}
M3 m3mul(const M3& A, const M3& B) {
  M3 R;
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 3; r++)
      R.m[c * 3 + r] = A.m[r] * B.m[c * 3] + A.m[3 + r] * B.m[c * 3 + 1] + A.m[6 + r] * B.m[c * 3 + 2];
  return R;
}
M3 m3inv(const M3& M) {  // the adjugate over the determinant
  auto a = [&](int c, int r) { return M.m[c * 3 + r]; };
  const float det = a(0, 0) * (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) -
                    a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
                    a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
  const float id = 1.0f / det;
  return M3{{(a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) * id, (a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2)) * id,
             (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1)) * id, (a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2)) * id,
             (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0)) * id, (a(1, 0) * a(0, 2) - a(0, 0) * a(1, 2)) * id,
             (a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1)) * id, (a(2, 0) * a(0, 1) - a(0, 0) * a(2, 1)) * id,
             (a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1)) * id}};
}
constexpr float kH = 0.5f;  // images.nim:5

// One level of minifyBy2 / magnifyBy2 from src into pre-pass buffer k.
const uint32_t* resample_level(const uint32_t* src, int64_t& w, int64_t& h, bool minify, int k) {
  const int64_t nw = minify ? (w + 1) / 2 : w * 2, nh = minify ? (h + 1) / 2 : h * 2;
  dev_grow(g.sm_buf[k], g.sm_cap[k], nw * nh);
  if (minify)
    launch_minify2(src, w, h, g.sm_buf[k], g.nsm, g.stream);
  else
    launch_magnify2(src, w, h, g.sm_buf[k], g.nsm, g.stream);
  w = nw;
  h = nh;
  return g.sm_buf[k];
}

void draw_transform(pxg_image* a, const pxg_image* b, M3 T, int blend) {
  const M3 inv0 = m3inv(T);
  V p = m3v(inv0, 0 + kH, 0 + kH);
  V dx = vsub(m3v(inv0, 1 + kH, 0 + kH), p);
  V dy = vsub(m3v(inv0, 0 + kH, 1 + kH), p);
  float filterBy2 = fnmax(vlen(dx), vlen(dy));
  // an infinite filterBy2 (a singular transform) would halve forever in the
  // reference's minify loop; raise instead
  if (std::isinf(filterBy2)) throw ApiError{"draw transform is not invertible"};
  const uint32_t* src = (const uint32_t*)b->data;
  int64_t bw = b->width, bh = b->height;
  int k = 0;
  while (filterBy2 >= 2.0f) {
    src = resample_level(src, bw, bh, true, k);
    k ^= 1;
    p = V{p.x / 2, p.y / 2};
    dx = V{dx.x / 2, dx.y / 2};
    dy = V{dy.x / 2, dy.y / 2};
    filterBy2 /= 2;
    T = m3mul(T, M3{{2, 0, 0, 0, 2, 0, 0, 0, 1}});
  }
  while (filterBy2 <= 0.5f) {
    if (bw * bh > ((int64_t)1 << 30)) throw ApiError{"draw would magnify the source image beyond 2^32 bytes"};
    src = resample_level(src, bw, bh, false, k);
    k ^= 1;
    p = V{p.x * 2, p.y * 2};
    dx = V{dx.x * 2, dx.y * 2};
    dy = V{dy.x * 2, dy.y * 2};
    filterBy2 *= 2;
    T = m3mul(T, M3{{1.0f / 2, 0, 0, 0, 1.0f / 2, 0, 0, 0, 1}});
  }
  const bool hasRotationOrScaling = !(dx.x == 1 && dx.y == 0 && dy.x == 0 && dy.y == 1);
  const bool smooth = !(vlen(dx) == 1.0f && vlen(dy) == 1.0f && frac_abs(T.m[6]) == 0.0f && frac_abs(T.m[7]) == 0.0f);
  if (!hasRotationOrScaling && !smooth) {
    launch_draw((uint32_t*)a->data, src, a->width, a->height, bw, bh, h_nim_i32(T.m[6]), h_nim_i32(T.m[7]), blend,
                g.tbl, g.nsm, g.stream);
    return;
  }
  // drawSmooth  images.nim:531-561
  const V c[4] = {m3v(T, 0, 0), m3v(T, (float)bw, 0), m3v(T, (float)bw, (float)bh), m3v(T, 0, (float)bh)};
  SmoothArgs G;
  for (int i = 0; i < 4; i++) {
    G.seg[i][0] = c[i].x;
    G.seg[i][1] = c[i].y;
    G.seg[i][2] = c[(i + 1) & 3].x;
    G.seg[i][3] = c[(i + 1) & 3].y;
  }
  const M3 inv = m3inv(T);
  const V sp = m3v(inv, 0 + kH, 0 + kH);
  const V sdx = vsub(m3v(inv, 1 + kH, 0 + kH), sp);
  const V sdy = vsub(m3v(inv, 0 + kH, 1 + kH), sp);
  G.px = sp.x;
  G.py = sp.y;
  G.dxx = sdx.x;
  G.dxy = sdx.y;
  G.dyx = sdy.x;
  G.dyy = sdy.y;
  int64_t yStart = a->height, yEnd = 0;
  for (int i = 0; i < 4; i++) {
    yStart = std::min<int64_t>(yStart, h_nim_int(floorf(c[i].y)));
    yEnd = std::max<int64_t>(yEnd, h_nim_int(ceilf(c[i].y)));
  }
  G.yStart = std::clamp<int64_t>(yStart, 0, a->height);
  G.yEnd = std::clamp<int64_t>(yEnd, 0, a->height);
  if (a->width > INT32_MAX) throw ApiError{"Image too wide for draw with a transform"};
  void* sc = scratch(smooth_scratch_bytes(a->width, G.yEnd - G.yStart));
  launch_draw_smooth((uint32_t*)a->data, a->width, a->height, src, bw, bh, G, blend, g.tbl, sc, g.nsm, g.stream);
}

pxg_image* resampled_copy(const pxg_image* im, int power, bool minify) {
  if (power < 0)
    throw ApiError{minify ? "Cannot minifyBy2 with negative power" : "Cannot magnifyBy2 with negative power"};
  int64_t w = im->width, h = im->height;
  for (int i = 0; i < power; i++) {
    w = minify ? (w + 1) / 2 : w * 2;
    h = minify ? (h + 1) / 2 : h * 2;
    if (w * h > ((int64_t)1 << 31)) throw ApiError{"Image too large"};
  }
  pxg_image* res = pxg_new_image(w, h);
  if (!res) throw ApiError{std::string(t_err)};
  const uint32_t* src = (const uint32_t*)im->data;
  w = im->width;
  h = im->height;
  int k = 0;
  for (int i = 0; i < power; i++) {
    if (i == power - 1) {  // the last level straight into the result
      if (minify)
        launch_minify2(src, w, h, (uint32_t*)res->data, g.nsm, g.stream);
      else
        launch_magnify2(src, w, h, (uint32_t*)res->data, g.nsm, g.stream);
    } else {
      src = resample_level(src, w, h, minify, k);
      k ^= 1;
    }
  }
  if (power == 0)
    CU(cudaMemcpyAsync(res->data, im->data, (size_t)(w * h * 4), cudaMemcpyDeviceToDevice, g.stream));
  return res;
}

// drawCorrect / drawTiled  images.nim:405-445, :680-683: every destination
// pixel samples the (pre-passed) source at inverseTransform * (x + h, y + h) - h
void draw_correct(pxg_image* a, const pxg_image* b, const M3& T, int blend, bool tiled) {
  M3 inv = m3inv(T);
  V p = m3v(inv, 0 + kH, 0 + kH);
  V dx = vsub(m3v(inv, 1 + kH, 0 + kH), p);
  V dy = vsub(m3v(inv, 0 + kH, 1 + kH), p);
  float filterBy2 = fnmax(vlen(dx), vlen(dy));
  if (std::isinf(filterBy2)) throw ApiError{"draw transform is not invertible"};
  const uint32_t* src = (const uint32_t*)b->data;
  int64_t bw = b->width, bh = b->height;
  int k = 0;
  while (filterBy2 >= 2.0f) {
    src = resample_level(src, bw, bh, true, k);
    k ^= 1;
    p = V{p.x / 2, p.y / 2};
    dx = V{dx.x / 2, dx.y / 2};
    dy = V{dy.x / 2, dy.y / 2};
    filterBy2 /= 2;
    inv = m3mul(M3{{0.5f, 0, 0, 0, 0.5f, 0, 0, 0, 1}}, inv);
  }
  while (filterBy2 <= 0.5f) {
    if (bw * bh > ((int64_t)1 << 30)) throw ApiError{"draw would magnify the source image beyond 2^32 bytes"};
    src = resample_level(src, bw, bh, false, k);
    k ^= 1;
    p = V{p.x * 2, p.y * 2};
    dx = V{dx.x * 2, dx.y * 2};
    dy = V{dy.x * 2, dy.y * 2};
    filterBy2 *= 2;
    inv = m3mul(M3{{2, 0, 0, 0, 2, 0, 0, 0, 1}}, inv);
  }
  Mat9 I;
  memcpy(I.m, inv.m, sizeof I.m);
  launch_draw_correct((uint32_t*)a->data, a->width, a->height, src, bw, bh, I, blend, tiled, g.tbl, g.nsm, g.stream);
}

// ---------------------------------------------------------------------------
// Non-solid paints: gradient fills (paints.nim:95-241) and the
// mask -> fill -> MaskBlend -> draw chain of fillPath / strokePath
// (paths.nim:2115-2142).  The per-paint geometry (the radial gradient's
// matrix, the edge angles) is float32 host arithmetic with the C library's
// atan2f / sinf / cosf, as the reference computes it once per paint.
// ---------------------------------------------------------------------------
inline float fix_angle_h(float a) {  // a float32 compared with the float64 PI
  const double pi = 3.141592653589793;
  const float tau = (float)(pi * 2);
  while ((double)a > pi) a -= tau;
  while ((double)a < -pi) a += tau;
  return a;
}
inline V vnorm(V v) {
  const float l = vlen(v);
  return V{v.x / l, v.y / l};
}

pxg_image temp_image(int i, int64_t w, int64_t h) {  // a zeroed non-owning scratch image
  dev_grow(g.pt_buf[i], g.pt_cap[i], w * h);
  CU(cudaMemsetAsync(g.pt_buf[i], 0, (size_t)(w * h * 4), g.stream));
  return pxg_image{(uint8_t*)g.pt_buf[i], w, h, 0};
}

void fill_gradient(pxg_image* im, const pxg_paint& p, float opacity) {
  const int nh = p.n_handles, ns = p.n_stops;
  if (nh < 0 || ns < 0 || (nh > 0 && !p.handles) || (ns > 0 && !p.stops)) throw ApiError{"Invalid gradient"};
  if (p.kind == 3 && nh != 2) throw ApiError{"Linear gradient requires 2 handles"};
  if (p.kind == 4 && nh != 3) throw ApiError{"Radial gradient requires 3 handles"};
  if (p.kind == 5 && nh != 3) throw ApiError{"Angular gradient requires 2 handles"};
  if (ns == 0) throw ApiError{"Gradient must have at least 1 color stop"};
  opacity = opacity < 0 ? 0 : (opacity > 1 ? 1 : opacity);
  if (opacity == 0) return;
  GradientArgs G{};
  G.kind = p.kind;
  G.nstops = ns;
  G.opacity = opacity;
  const V h0{p.handles[0], p.handles[1]}, h1{p.handles[2], p.handles[3]};
  if (p.kind == 3) {
    const V d = vsub(h1, h0);
    G.atx = h0.x;
    G.aty = h0.y;
    G.dx = d.x;
    G.dy = d.y;
    G.det = d.x * d.x + d.y * d.y;
  } else if (p.kind == 4) {
    const V skew{p.handles[4], p.handles[5]};
    const float distanceX = vlen(vsub(h0, h1)), distanceY = vlen(vsub(h0, skew));
    const V n = vnorm(vsub(h0, h1));
    const float ang = fix_angle_h(atan2f(n.y, n.x));
    const float sn = sinf(ang), cs = cosf(ang);
    const M3 T{{1, 0, 0, 0, 1, 0, h0.x, h0.y, 1}}, R{{cs, sn, 0, -sn, cs, 0, 0, 0, 1}};
    const M3 S{{distanceX, 0, 0, 0, distanceY, 0, 0, 0, 1}};
    const M3 inv = m3inv(m3mul(m3mul(T, R), S));
    memcpy(G.m, inv.m, sizeof G.m);
  } else {
    const V n = vnorm(vsub(h1, h0));
    G.cx = h0.x;
    G.cy = h0.y;
    G.gradientAngle = fix_angle_h(atan2f(n.y, n.x));
  }
  dev_grow(g.pt_stops, g.pt_stops_cap, 5 * (long long)ns);
  CU(cudaMemcpyAsync(g.pt_stops, p.stops, sizeof(float) * 5 * (size_t)ns, cudaMemcpyHostToDevice, g.stream));
  launch_gradient((uint32_t*)im->data, im->width, im->height, G, g.pt_stops, g.nsm, g.stream);
}

void check_paint(const pxg_paint* p) {
  if (!p) throw ApiError{"paint is null"};
  if (p->kind < 0 || p->kind > 5) throw ApiError{"Invalid paint kind"};
  check_blend(p->blend_mode);
  if ((p->kind == 1 || p->kind == 2)) {
    if (!p->image) throw ApiError{"Image paint needs an image"};
    check_image(p->image);
  }
}

// the paint's own image at opacity 1  paths.nim:2121-2134
void paint_fill_image(pxg_image* fill, const pxg_paint& p) {
  M3 m;
  memcpy(m.m, p.image_mat, sizeof m.m);
  if (p.kind == 1)
    draw_transform(fill, p.image, m, 0);
  else if (p.kind == 2)
    draw_correct(fill, p.image, m, 0, true);
  else
    fill_gradient(fill, p, 1.0f);
}

// images.nim:261-277
void apply_opacity(pxg_image* im, float opacity) {
  const uint32_t o = (uint16_t)h_nim_i32(roundf(255 * opacity));
  if (o == 255) return;
  if (o == 0) {
    CU(cudaMemsetAsync(im->data, 0, (size_t)(im->width * im->height * 4), g.stream));
    return;
  }
  launch_apply_opacity((uint32_t*)im->data, im->width * im->height, o, g.nsm, g.stream);
}

// fill.draw(mask, MaskBlend); image.draw(fill, blendMode)  paths.nim:2136-2142
void composite_paint(pxg_image* im, pxg_image* mask, const pxg_paint& p) {
  pxg_image fill = temp_image(1, im->width, im->height);
  paint_fill_image(&fill, p);
  const float op = p.opacity < 0 ? 0 : (p.opacity > 1 ? 1 : p.opacity);
  if (op != 1) apply_opacity(mask, op);
  const int64_t W = im->width, H = im->height;
  launch_draw((uint32_t*)fill.data, (const uint32_t*)mask->data, W, H, W, H, 0, 0, kMask, g.tbl, g.nsm, g.stream);
  launch_draw((uint32_t*)im->data, (const uint32_t*)fill.data, W, H, W, H, 0, 0, p.blend_mode, g.tbl, g.nsm,
              g.stream);
}
}  // namespace

extern "C" {

int pxg_image_draw_transform(pxg_image* a, const pxg_image* b, const float* mat3, int blend) {
  return guarded_images({a, b}, [&] {
    check_image(a);
    check_image(b);
    check_blend(blend);
    if (!mat3) throw ApiError{"transform is null"};
    M3 T;
    memcpy(T.m, mat3, sizeof(T.m));
    Timed t;
    draw_transform(a, b, T, blend);
    CU(cudaGetLastError());
    t.done();
  });
}

static pxg_image* resampled(const pxg_image* im, int power, bool minify) {
  pxg_image* out = nullptr;
  guarded([&] {
    check_image(im);
    Timed t;
    pxg_image* res = resampled_copy(im, power, minify);
    if (cudaGetLastError() != cudaSuccess) {
      pxg_image_free(res);
      throw ApiError{"CUDA error in minifyBy2/magnifyBy2"};
    }
    t.done();
    out = res;
  });
  return out;
}
pxg_image* pxg_image_minify_by2(const pxg_image* im, int power) { return resampled(im, power, true); }
pxg_image* pxg_image_magnify_by2(const pxg_image* im, int power) { return resampled(im, power, false); }

int pxg_image_draw_tiled(pxg_image* a, const pxg_image* b, const float* mat3, int blend) {
  return guarded([&] {
    check_image(a);
    check_image(b);
    check_blend(blend);
    if (!mat3) throw ApiError{"transform is null"};
    M3 T;
    memcpy(T.m, mat3, sizeof(T.m));
    Timed t;
    draw_correct(a, b, T, blend, true);
    CU(cudaGetLastError());
    t.done();
  });
}

int pxg_image_fill_path_paint(pxg_image* im, const float* cmds, int64_t n, const pxg_paint* paint,
                              const float* transform, int winding) {
  return guarded([&] {
    check_image(im);
    check_paint(paint);
    const float op = paint->opacity < 0 ? 0 : (paint->opacity > 1 ? 1 : paint->opacity);
    if (op == 0) return;  // paths.nim:2101-2104
    if (paint->kind == 0) {
      if (pxg_image_fill_path(im, cmds, n, paint->color, paint->opacity, paint->blend_mode, transform, winding) != 0)
        throw ApiError{std::string(t_err)};
      return;
    }
    pxg_image mask = temp_image(0, im->width, im->height);
    static const float white[4] = {1, 1, 1, 1};
    if (pxg_image_fill_path(&mask, cmds, n, white, 1, 0, transform, winding) != 0) throw ApiError{std::string(t_err)};
    Timed t;
    composite_paint(im, &mask, *paint);
    CU(cudaGetLastError());
    t.done();
  });
}

int pxg_image_stroke_path_paint(pxg_image* im, const float* cmds, int64_t n, const pxg_paint* paint,
                                const float* transform, float width, int cap, int join, float miterLimit,
                                const float* dashes, int64_t nd) {
  return guarded([&] {
    check_image(im);
    check_paint(paint);
    const float op = paint->opacity < 0 ? 0 : (paint->opacity > 1 ? 1 : paint->opacity);
    if (op == 0) return;
    if (paint->kind == 0) {
      if (pxg_image_stroke_path(im, cmds, n, paint->color, paint->opacity, paint->blend_mode, transform, width, cap,
                                join, miterLimit, dashes, nd) != 0)
        throw ApiError{std::string(t_err)};
      return;
    }
    pxg_image mask = temp_image(0, im->width, im->height);
    static const float white[4] = {1, 1, 1, 1};
    if (pxg_image_stroke_path(&mask, cmds, n, white, 1, 0, transform, width, cap, join, miterLimit, dashes, nd) != 0)
      throw ApiError{std::string(t_err)};
    Timed t;
    composite_paint(im, &mask, *paint);
    CU(cudaGetLastError());
    t.done();
  });
}

// applyOpacity  images.nim:261-277
int pxg_image_apply_opacity(pxg_image* im, float opacity) {
  return guarded_images({im}, [&] {
    check_image(im);
    Timed t;
    apply_opacity(im, opacity);
    CU(cudaGetLastError());
    t.done();
  });
}

// fill(image, paint)  pixie.nim:120-131
int pxg_image_fill_paint(pxg_image* im, const pxg_paint* paint) {
  return guarded([&] {
    check_image(im);
    check_paint(paint);
    if (paint->kind == 0) {
      if (pxg_image_fill(im, paint->color) != 0) throw ApiError{std::string(t_err)};
      return;
    }
    if (paint->kind == 1 || paint->kind == 2) {
      CU(cudaMemsetAsync(im->data, 0, (size_t)(im->width * im->height * 4), g.stream));
      const float w = (float)im->width, h = (float)im->height;
      const float rect[] = {1, 0, 0, 2, w, 0, 2, w, h, 2, 0, h, 0};  // Move, Line x3, Close
      if (pxg_image_fill_path_paint(im, rect, 13, paint, nullptr, 0) != 0) throw ApiError{std::string(t_err)};
      return;
    }
    Timed t;
    fill_gradient(im, *paint, paint->opacity);
    CU(cudaGetLastError());
    t.done();
  });
}

int pxg_image_blur(pxg_image* im, float radius, const float* oob) {
  return guarded_images({im}, [&] {
    check_image(im);
    int64_t r = nim_round_int(radius);  // images.nim:308-312
    if (r == 0) return;
    if (r < 0) throw ApiError{"Cannot apply negative blur"};
    if (r > (1 << 20)) throw ApiError{"Blur radius too large"};
    static const float zero[4] = {0, 0, 0, 0};
    uint32_t o = color_to_rgbx(oob ? oob : zero);
    weights_for(r);
    // an image-sized buffer for the small-radius kernels, the tensor-core
    // passes' padded intermediate for the others: one size serves both
    const long long tmp_bytes = blur_scratch_bytes(im->width, im->height);
    uint32_t* tmp = (uint32_t*)scratch(tmp_bytes);
    Timed t;
    // an image the library allocated, whose address nobody holds, may take
    // the fused small-radius kernel: the result lands in the scratch buffer
    // and the two buffers change owners (stream order keeps every earlier
    // and later use of either buffer in place)
    const bool swap_ok = im->owned && !im->exported;
    if (blur_dispatch((uint32_t*)im->data, tmp, tmp_bytes, im->width, im->height, r, o, swap_ok)) {
      std::swap(im->data, g.scratch);
      std::swap(im->cap, g.scratch_cap);
    }
    CU(cudaGetLastError());
    t.done();
    if (g.blocking) check_device_error();
  });
}

int pxg_image_spread(pxg_image* im, float spread) {
  return guarded([&] {
    check_image(im);
    int64_t s = nim_round_int(spread);
    if (s == 0) return;
    if (s > (1 << 24) || s < -(1 << 24)) throw ApiError{"Spread too large"};
    long long n = im->width * im->height;
    uint8_t* a = (uint8_t*)scratch(2 * n);
    Timed t;
    launch_spread((uint32_t*)im->data, a, a + n, im->width, im->height, (int)s, g.nsm, g.stream);
    CU(cudaGetLastError());
    t.done();
  });
}

int pxg_image_shadow_into(const pxg_image* im, pxg_image* res, float ox, float oy, float spread,
                          float blur, const float* color) {
  return guarded_images({im, res}, [&] {
    check_image(im);
    check_image(res);
    if (res->width != im->width || res->height != im->height)
      throw ApiError{"Shadow output must have the size of the image"};
    int64_t s = nim_round_int(spread), r = nim_round_int(blur);
    if (r < 0) throw ApiError{"Cannot apply negative blur"};
    if (r > (1 << 20) || s > (1 << 24) || s < -(1 << 24)) throw ApiError{"Shadow parameters too large"};
    long long n = im->width * im->height;
    const uint16_t* kern = r > 0 ? weights_for(r) : nullptr;
    Timed t;
    const uint32_t* src = (const uint32_t*)im->data;
    if (ox != floorf(ox) || oy != floorf(oy)) {
      // mask.draw(image, translate(offset), OverwriteBlend) takes drawSmooth
      // (images.nim:768-769); the shadow then runs on that mask at offset 0
      pxg_image mask = temp_image(0, im->width, im->height);
      draw_transform(&mask, im, M3{{1, 0, 0, 0, 1, 0, ox, oy, 1}}, kOverwrite);
      src = (const uint32_t*)mask.data;
      ox = 0;
      oy = 0;
    }
    uint8_t* a = (uint8_t*)scratch(2 * n);  // after the smooth draw, which uses the scratch too
    launch_shadow(src, (uint32_t*)res->data, a, a + n, im->width, im->height, (long long)ox, (long long)oy, (int)s,
                  (int)r, kern, color_to_rgbx(color), g.nsm, g.stream);
    CU(cudaGetLastError());
    t.done();
  });
}

pxg_image* pxg_image_shadow(const pxg_image* im, float ox, float oy, float spread, float blur,
                            const float* color) {
  pxg_image* out = nullptr;
  guarded([&] {
    check_image(im);
    pxg_image* res = pxg_new_image(im->width, im->height);
    if (!res) throw ApiError{std::string(t_err)};
    if (pxg_image_shadow_into(im, res, ox, oy, spread, blur, color) != 0) {
      std::string m(t_err);
      pxg_image_free(res);
      throw ApiError{m};
    }
    out = res;
  });
  return out;
}

int pxg_blend_pixels(int blend, const void* bd, const void* src, void* out, int64_t n) {
  return guarded([&] {
    check_blend(blend);
    launch_blend_pixels(blend, g.tbl, (const uint32_t*)bd, (const uint32_t*)src, (uint32_t*)out, n,
                        g.stream);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(g.stream));
  });
}

}  // extern "C"
