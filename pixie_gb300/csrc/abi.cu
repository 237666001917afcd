// The C ABI of include/pxg.h: device context, image handles, the fill/stroke
// job runner and the image operations.  No C++ exception crosses the ABI;
// failures set a per-thread message returned by pxg_take_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pxg.h"
#include "host_geom.h"
#include "pxg_device.cuh"
#include "raster.cuh"

struct pxg_image {
  uint8_t* data;
  int64_t width, height;
  int owned;
};

namespace pxg {
__global__ void k_setup(PathJob* jobs, Arena A, int maxBands);
__global__ void k_rows(PathJob* jobs, int njobs, Arena A, const uint8_t* tbl, long long totalRows);
__global__ void k_rows_wide(PathJob* jobs, Arena A, const uint8_t* tbl);
__global__ void k_xclears(PathJob* jobs, Arena A);
size_t rows_smem_fast();
size_t rows_smem_wide();
int rows_warps_fast();
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
  uint8_t* tbl = nullptr;
  // fill arena
  float4* segs = nullptr;
  int* segw = nullptr;
  long long seg_cap = 0, segw_cap = 0;
  uint2* segband = nullptr;
  long long segband_cap = 0;
  Band* bands = nullptr;
  long long band_cap = 0;
  long long* ovf = nullptr;
  long long ovf_cap = 0;
  long long* xcl = nullptr;
  long long xcl_cap = 0;
  // upload area: jobs | counters | prims (device and pinned mirror)
  unsigned char* d_up = nullptr;
  unsigned char* h_up = nullptr;
  size_t up_cap = 0;
  // misc scratch
  uint16_t* kern = nullptr;
  long long kern_cap = 0;
  unsigned char* scratch = nullptr;
  long long scratch_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0;
  bool blocking = true;  // image operations wait for their GPU work
  std::map<int64_t, uint16_t*> weights;  // gaussian weights per radius, on the device
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
  std::vector<uint8_t> t(65536);
  straight_alpha_table(t.data());
  CU(cudaMalloc(&g.tbl, 65536));
  CU(cudaMemcpy(g.tbl, t.data(), 65536, cudaMemcpyHostToDevice));
  CU(cudaFuncSetAttribute(k_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem_fast()));
  CU(cudaFuncSetAttribute(k_rows_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem_wide()));
  g.setupSmemMax = allow_max_smem((const void*)k_setup);
  g.blurSmemMax = std::min(allow_max_smem((const void*)k_blur_x), allow_max_smem((const void*)k_blur_y));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem((const void*)k_blurf_x));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem((const void*)k_blurf_y));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem(blurb_kernel(true)));
  g.blurSmemMax = std::min(g.blurSmemMax, allow_max_smem(blurb_kernel(false)));
  CU(cudaEventCreate(&g.ev0));
  CU(cudaEventCreate(&g.ev1));
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
  return d;
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

// Runs fill jobs whose primitives are already in `prims` (job.prim_off set).
// Jobs must target distinct images: a job whose workspace ran out is rerun
// alone, after the others were drawn.  Returns per-job status.
void run_jobs(std::vector<PathJob>& jobs, const std::vector<Prim>& prims, std::vector<int>& status) {
  const int nj = (int)jobs.size();
  status.assign((size_t)nj, kOk);
  std::vector<int> todo(nj);
  for (int i = 0; i < nj; i++) todo[i] = i;
  long long seg_need = std::max<long long>(1 << 16, (long long)prims.size() * 8);
  for (int attempt = 0; attempt < 12 && !todo.empty(); attempt++) {
    std::vector<PathJob> run;
    long long rows = 0, maxH = 1;
    for (int i : todo) {
      PathJob j = jobs[i];
      j.row_off = rows;
      rows += j.H;
      maxH = std::max<long long>(maxH, j.H);
      j.status = kOk;
      run.push_back(j);
    }
    const int nr = (int)run.size();
    const int maxBands = (int)(std::max<long long>(1, maxH / 4) + 1);
    const size_t setupSmem = (size_t)maxBands * 8;
    if (setupSmem > g.setupSmemMax) throw ApiError{"Image too tall for the fill kernels"};

    dev_grow(g.segs, g.seg_cap, seg_need);
    dev_grow(g.segw, g.segw_cap, g.seg_cap);
    dev_grow(g.segband, g.segband_cap, g.seg_cap);
    dev_grow(g.bands, g.band_cap, (long long)nr * maxBands);
    dev_grow(g.ovf, g.ovf_cap, rows);
    dev_grow(g.xcl, g.xcl_cap, 3 * (2 * rows + 1024));

    const size_t jobsBytes = align_up(sizeof(PathJob) * nr, 256);
    const size_t ctrBytes = 256;
    const size_t primBytes = sizeof(Prim) * std::max<size_t>(prims.size(), 1);
    const size_t need = jobsBytes + ctrBytes + primBytes;
    if (need > g.up_cap) {
      if (g.d_up) cudaFree(g.d_up);
      if (g.h_up) cudaFreeHost(g.h_up);
      g.d_up = nullptr;
      g.h_up = nullptr;
      size_t cap = std::max(need, g.up_cap * 2);
      CU(cudaMalloc(&g.d_up, cap));
      CU(cudaMallocHost(&g.h_up, cap));
      g.up_cap = cap;
    }
    memcpy(g.h_up, run.data(), sizeof(PathJob) * nr);
    memset(g.h_up + jobsBytes, 0, ctrBytes);
    if (!prims.empty()) memcpy(g.h_up + jobsBytes + ctrBytes, prims.data(), sizeof(Prim) * prims.size());
    CU(cudaMemcpyAsync(g.d_up, g.h_up, need, cudaMemcpyHostToDevice, g.stream));

    PathJob* dj = reinterpret_cast<PathJob*>(g.d_up);
    Arena A;
    A.prims = reinterpret_cast<const Prim*>(g.d_up + jobsBytes + ctrBytes);
    A.segs = g.segs;
    A.segw = g.segw;
    A.seg_cap = g.seg_cap;
    A.segband = g.segband;
    A.bands = g.bands;
    A.band_cap = g.band_cap;
    A.counters = reinterpret_cast<unsigned long long*>(g.d_up + jobsBytes);
    A.ovf_rows = g.ovf;
    A.ovf_cap = g.ovf_cap;
    A.xclears = g.xcl;
    A.xclear_cap = g.xcl_cap / 3;

    k_setup<<<nr, 256, setupSmem, g.stream>>>(dj, A, maxBands); note_launch();
    CU(cudaGetLastError());
    const int wpb = rows_warps_fast();
    long long blocks = (rows + wpb - 1) / wpb;
    blocks = std::min<long long>(blocks, (long long)g.nsm * 16);
    blocks = std::max<long long>(blocks, 1);
    k_rows<<<(unsigned)blocks, wpb * 32, rows_smem_fast(), g.stream>>>(dj, nr, A, g.tbl, rows); note_launch();
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(g.h_up, g.d_up, jobsBytes + ctrBytes, cudaMemcpyDeviceToHost, g.stream));
    CU(cudaStreamSynchronize(g.stream));
    unsigned long long ctr[kNumCounters];
    memcpy(ctr, g.h_up + jobsBytes, sizeof ctr);
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
      CU(cudaMemcpyAsync(g.h_up, g.d_up, jobsBytes, cudaMemcpyDeviceToHost, g.stream));
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
    if (grow) {
      seg_need = std::max<long long>(seg_need * 4, (long long)ctr[kCtrSegs] * 2);
    }
    todo = again;
  }
  for (int i : todo) status[(size_t)i] = kErrArenaFull;
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
  j.img = img->data;
  j.W = img->width;
  j.H = img->height;
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

template <class F>
int guarded(F&& f) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  try {
    ensure_init();
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
  return guarded([&] { CU(cudaStreamSynchronize(g.stream)); });
}

float pxg_last_gpu_ms(void) { return g.last_ms; }

int pxg_set_blocking(int blocking) {
  return guarded([&] { g.blocking = blocking != 0; });
}

int64_t pxg_launch_count(void) { return (int64_t)launch_count(); }

pxg_image* pxg_new_image(int64_t width, int64_t height) {
  pxg_image* out = nullptr;
  guarded([&] {
    if (width <= 0 || height <= 0) throw ApiError{"Image width and height must be > 0"};
    pxg_image* im = new pxg_image{nullptr, width, height, 1};
    cudaError_t e = cudaMalloc((void**)&im->data, (size_t)(width * height * 4));
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
  if (im->owned && im->data) cudaFree(im->data);
  delete im;
}

int64_t pxg_image_width(const pxg_image* im) { return im ? im->width : 0; }
int64_t pxg_image_height(const pxg_image* im) { return im ? im->height : 0; }
void* pxg_image_device_ptr(pxg_image* im) { return im ? im->data : nullptr; }

int pxg_image_upload(pxg_image* im, const void* host, int64_t nbytes) {
  return guarded([&] {
    check_image(im);
    if (nbytes != im->width * im->height * 4) throw ApiError{"Byte count does not match the image"};
    CU(cudaMemcpyAsync(im->data, host, (size_t)nbytes, cudaMemcpyHostToDevice, g.stream));
    CU(cudaStreamSynchronize(g.stream));
  });
}

int pxg_image_download(const pxg_image* im, void* host, int64_t nbytes) {
  return guarded([&] {
    check_image(im);
    if (nbytes != im->width * im->height * 4) throw ApiError{"Byte count does not match the image"};
    CU(cudaMemcpyAsync(host, im->data, (size_t)nbytes, cudaMemcpyDeviceToHost, g.stream));
    CU(cudaStreamSynchronize(g.stream));
  });
}

int pxg_image_fill(pxg_image* im, const float* color) {
  return guarded([&] {
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

int pxg_image_draw(pxg_image* a, const pxg_image* b, int64_t tx, int64_t ty, int blend) {
  return guarded([&] {
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

static int64_t nim_round_int(float v) {
  float r = roundf(v);
  if (!(r >= -9223372036854775808.0f && r < 9223372036854775808.0f)) return INT64_MIN;
  return (int64_t)r;
}

int pxg_image_blur(pxg_image* im, float radius, const float* oob) {
  return guarded([&] {
    check_image(im);
    int64_t r = nim_round_int(radius);  // images.nim:308-312
    if (r == 0) return;
    if (r < 0) throw ApiError{"Cannot apply negative blur"};
    if (r > (1 << 20)) throw ApiError{"Blur radius too large"};
    static const float zero[4] = {0, 0, 0, 0};
    uint32_t o = color_to_rgbx(oob ? oob : zero);
    const uint16_t* kern = weights_for(r);
    uint32_t* tmp = (uint32_t*)scratch(im->width * im->height * 4);
    Timed t;
    launch_blur((uint32_t*)im->data, tmp, im->width, im->height, (int)r, kern, o, g.nsm,
                g.blurSmemMax, g.stream);
    CU(cudaGetLastError());
    t.done();
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
  return guarded([&] {
    check_image(im);
    check_image(res);
    if (res->width != im->width || res->height != im->height)
      throw ApiError{"Shadow output must have the size of the image"};
    if (ox != floorf(ox) || oy != floorf(oy))
      throw ApiError{"Shadow offsets must be whole pixels (the smooth draw path is not provided)"};
    int64_t s = nim_round_int(spread), r = nim_round_int(blur);
    if (r < 0) throw ApiError{"Cannot apply negative blur"};
    if (r > (1 << 20) || s > (1 << 24) || s < -(1 << 24)) throw ApiError{"Shadow parameters too large"};
    long long n = im->width * im->height;
    uint8_t* a = (uint8_t*)scratch(2 * n);
    const uint16_t* kern = r > 0 ? weights_for(r) : nullptr;
    Timed t;
    launch_shadow((const uint32_t*)im->data, (uint32_t*)res->data, a, a + n, im->width, im->height,
                  (long long)ox, (long long)oy, (int)s, (int)r, kern, color_to_rgbx(color), g.nsm,
                  g.stream);
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
