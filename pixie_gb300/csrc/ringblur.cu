// Gaussian blur passes on the tensor cores: TMA-fed rows, the f16 input ring
// in tensor memory, transposed outputs.
//
// One pass of pixie's blur (images.nim:304-365) is, per channel,
//   out[x] = (sum_t w[t] * p[x - r + t]) div 256 div 255,   t = 0 .. 2r,
// with taps outside the image reading the outOfBounds colour.  Both passes
// here run along the rows of their input and write their output transposed,
// as the reference's X pass stores blurX: pass 1 reads the image's rows and
// writes the intermediate (W rows of H pixels), pass 2 reads the
// intermediate's rows (the image's columns) and writes the image back in its
// own orientation.  For a tile of 64 outputs along a row and the K = 64 + 2r
// inputs they read, a pass is D[m][n] = sum_k A[m][k] * B[n][k] with the
// banded (Toeplitz) matrix B[n][k] = w[k - n]; a row m = 4 j + c of A is
// channel c of line j (an input row), 32 lines per band.
//
// Exactness.  A holds each 8-bit channel value v as the f16 subnormal
// v * 2^-24 (its bit pattern is v itself); B holds integer weights, split into
// bytes (w = 256 wh + wl: one MMA of N = 128 whose B rows 0..63 hold wh and
// 64..127 hold wl) unless every weight of the radius is an exact f16.  Every product is an integer times 2^-24, every sum a multiple
// of 2^-24 below 1, exact in the f32 accumulator.  The epilogue forms
// S * 2^-24 (S the reference's integer sum) and takes
// floor(S / 65280) = floor(S * C) with C = 1/65280 rounded up to float32,
// which is exact for every S < 2^24 (checked exhaustively on the host): one
// fused multiply-add rounding toward minus infinity onto 1.5 * 2^23 leaves the
// quotient in the low byte of the result.
//
// Pipeline (one CTA per SM, persistent over work items = (band of 32 lines,
// segment of the row)):
//   warp 0      TMA: input chunks of 64 positions x 32 lines into raw stages
//               in shared memory
//   8 warps     two groups of four on alternate chunks: each thread converts
//               its (line, channel) row of the chunk to f16 and stores it into
//               the ring in tensor memory (tcgen05.st; the warp's lane quarter
//               holds its rows), so each input pixel is converted once and
//               consecutive tiles share their halo there
//   1 warp      issues the MMAs of a tile: A from the tensor-memory ring (the
//               K span may wrap; each 16-wide K step lies inside the ring), B
//               (weights) from shared memory, 128-byte swizzled; then frees
//               the ring chunk that later tiles no longer read.  The whole warp
//               runs the loop with uniform operands; one elected lane issues.
//   8 warps     epilogue, two groups of four on alternate tiles: TMEM ->
//               quotient bytes -> a 4 x 4 byte transpose across each quad of
//               lanes (the four channels of a line) -> whole pixels, staged
//               transposed in 128-byte-swizzled shared memory (64 rows of 32
//               pixels) and written with one TMA store per tile (the group's
//               first thread issues it after a group barrier)
// The operand traffic of the MMAs is then the weights only (2 KB per
// 128 x 64 x 16 step, 4 KB per 128 x 128 x 16 step), below the tensor core's
// math time.  The intermediate's rows are padded (ring_tmp_pitch) and work
// items are planned over all SMs (plan_pass).  Every mbarrier wait is
// bounded; a role whose wait runs out sets *err and stops; the others then
// run out too, in-flight copies, MMAs and stores are waited for (bounded),
// and the CTA frees its tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>

#include "pxg_device.cuh"
#include "tc_ptx.cuh"

namespace pxg {

void note_launch();

// Converter trace (a diagnostic, off unless pxg_ring_trace enables it): for
// CTA 0 and the second warp of each converter group, the clock64 of every
// ring chunk before its barrier waits, after them, and after its
// tensor-memory stores -- where a pass's time goes between the roles.
// (The trace's never-taken branch in the converter loop is also what lets the
// compiler keep that loop's bookkeeping on the uniform datapath: without it
// a 4096 x 4096 blur measured 25 % slower, with 3x the branch and 1/50 of the
// uniform-pipe instructions.)
constexpr int kTraceChunks = 256;
__device__ int g_ring_trace_on;
__device__ long long g_ring_trace[2][kTraceChunks][3];

namespace {

using namespace tc;

constexpr int kConvWarps = 8;             // two converter groups of four warps
constexpr int kEpiWarps = 8;              // two epilogue groups of four warps
constexpr int kMmaWarp = 1 + kConvWarps;  // warp 0 issues the TMA loads
constexpr int kEpiWarp0 = kMmaWarp + 1;
constexpr int kRingThreads = 32 * (kEpiWarp0 + kEpiWarps);  // 576
constexpr int kLines = 32;       // lines per band (x 4 channels = MMA M of 128)
constexpr int kPos = 64;         // positions per input chunk = outputs per tile (MMA N)
constexpr int kRawW = kPos + 4;  // raw box width: 16-byte aligned start, rows of 272 bytes
constexpr int kMaxAcc = 4;       // TMEM accumulators (two with byte-split weights)
constexpr int kMaxRaw = 12;      // raw stages (upper bound)
constexpr int kMaxRing = 8;      // ring chunks (upper bound)
constexpr int kTmemCols = 512;
constexpr int kRingCol0 = 256;   // accumulators in columns [0, 256), the ring above
constexpr uint32_t kBBlockBytes = kPos * 128;  // 64 weight rows x 64 positions (f16), 8 atoms
constexpr float kQuotC24 = 257.00394f;         // RU(1/65280) * 2^24, exactly
constexpr float kMagic = 12582912.0f;          // 1.5 * 2^23

struct RingArgs {
  int alen, clen;  // input row length (pass axis) and number of rows (lines)
  int opitch;      // pixels between consecutive output rows (>= clen)
  int r;
  int kspan;       // K span of a tile: 64 + 2r rounded up to 16
  int nring;       // ring chunks (ring positions = 64 * nring)
  int nraw;        // raw stages
  int rawStride;   // bytes between raw stages
  int delta;       // input offset of a chunk inside its 16-byte aligned box
  int seglen;      // outputs per segment (multiple of 64)
  int nseg;        // segments per band
  long long nitems;
  uint32_t oob;
};

constexpr int kRawBytes = kLines * kRawW * 4;

// Shared-memory layout (offsets from a 1024-aligned base).
// An epilogue group's output tile staged for its TMA store: 64 positions (box
// rows) x 32 lines (128 bytes, 128-byte swizzled); two per group.
constexpr uint32_t kStageBytes = kPos * kLines * 4;

struct RingSmem {
  uint32_t raw, bhi, stage, bars, total;
};
__host__ __device__ inline RingSmem ring_smem(const RingArgs& a, bool split) {
  RingSmem s;
  s.raw = 0;
  const uint32_t bBytes = (uint32_t)((a.kspan + 63) / 64) * kBBlockBytes;
  s.bhi = (uint32_t)a.nraw * a.rawStride;  // B: 64 rows per K block (128 with byte-split weights)
  s.stage = s.bhi + (split ? 2 : 1) * bBytes;  // 1024-aligned: every region above is a multiple of 1 KB
  s.bars = s.stage + 4 * kStageBytes;
  s.total = s.bars + (2 * kMaxRaw + 2 * kMaxRing + 2 * kMaxAcc + 1) * 8 + 16;
  return s;
}

// Channel c of pixels x and y as the f16 subnormals x_c * 2^-24, y_c * 2^-24.
__device__ __forceinline__ uint32_t sub_pair(uint32_t x, uint32_t y, uint32_t sel) {
  return __byte_perm(x, y, sel) & 0x00FF00FFu;
}

__device__ __forceinline__ void item_geom(const RingArgs& a, long long it, int& band, int& s0, int& T,
                                          int& nch) {
  band = (int)(it / a.nseg);
  s0 = (int)(it % a.nseg) * a.seglen;
  const int len = min(a.seglen, a.alen - s0);
  T = (len + kPos - 1) / kPos;
  nch = (kPos * (T - 1) + a.kspan + kPos - 1) / kPos;
}

// 16 columns of this warp's TMEM lane quarter from registers.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};\n" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
      "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
      : "memory");
}

// MMA with A in tensor memory (M rows in the lanes, K packed two f16 per
// column) and B from shared memory; issued by one elected lane of the warp.
__device__ __forceinline__ void mma_ts_elect(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred e, p;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "@e tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// DELTA = (first input position of a chunk) mod 4 = (-r) mod 4, the pixel
// offset of the chunk inside its 16-byte aligned box, fixed per radius: as a
// template parameter the converters' word selection is straight-line code.
template <bool SPLIT, int DELTA>
__global__ void __launch_bounds__(kRingThreads, 1)
    k_blur_ring(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout, const RingArgs a,
                const uint16_t* __restrict__ kern, int* err, int late) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  constexpr int kAcc = SPLIT ? 2 : 4;
  constexpr int accCols = SPLIT ? 2 * kPos : kPos;  // TMEM columns per accumulator
  const RingSmem L = ring_smem(a, SPLIT);
  // the warp index through a shuffle, so the compiler knows it is warp-uniform
  // (each role's loop then runs on the uniform datapath)
  const int tid = threadIdx.x, warp = __shfl_sync(0xffffffffu, tid >> 5, 0), lane = tid & 31;
  const uint32_t base = smem_u32(sm);
  const uint32_t rawFull = base + L.bars, rawEmpty = rawFull + 8 * kMaxRaw, ringFull = rawEmpty + 8 * kMaxRaw,
                 ringEmpty = ringFull + 8 * kMaxRing, tFull = ringEmpty + 8 * kMaxRing, tEmpty = tFull + 8 * kMaxAcc,
                 doneBar = tEmpty + 8 * kMaxAcc;
  uint32_t* taddr_s =
      reinterpret_cast<uint32_t*>(sm + L.bars + (2 * kMaxRaw + 2 * kMaxRing + 2 * kMaxAcc + 1) * 8);
  const int r = a.r;
  const bool trace = g_ring_trace_on != 0;
  if (late) pdl_trigger();  // the next pass may be set up while this one runs (else after the start-wait)

  // The Toeplitz weights, once per CTA (K padded with zeros to whole blocks).
  const int kpad = (a.kspan + 63) / 64 * 64;
  for (int i = tid; i < kPos * kpad; i += kRingThreads) {
    const int n = i / kpad, k = i - n * kpad, t = k - n;
    const uint32_t w = (t >= 0 && t <= 2 * r) ? kern[t] : 0u;
    if (SPLIT) {
      // one 128-row operand per K block: the high weight bytes in rows 0..63,
      // the low bytes in rows 64..127, so one MMA of N = 128 forms both sums
      // (accumulator columns [0, 64) and [64, 128))
      *reinterpret_cast<uint16_t*>(sm + L.bhi + sw128_off(n, k, 2 * kBBlockBytes)) = f16_bits(w >> 8);
      *reinterpret_cast<uint16_t*>(sm + L.bhi + sw128_off(kPos + n, k, 2 * kBBlockBytes)) = f16_bits(w & 255u);
    } else {
      *reinterpret_cast<uint16_t*>(sm + L.bhi + sw128_off(n, k, kBBlockBytes)) = f16_bits(w);
    }
  }
  if (tid == 0) {
    for (int b = 0; b < kMaxRaw; b++) {
      mbar_init(rawFull + 8 * b, 1);
      mbar_init(rawEmpty + 8 * b, kConvWarps / 2);  // one lane of each converter warp of a group
    }
    for (int b = 0; b < kMaxRing; b++) {
      mbar_init(ringFull + 8 * b, kConvWarps / 2);
      mbar_init(ringEmpty + 8 * b, 1);
    }
    for (int b = 0; b < kMaxAcc; b++) {
      mbar_init(tFull + 8 * b, 1);
      mbar_init(tEmpty + 8 * b, kEpiWarps / 2);  // one lane of each epilogue warp of a group
    }
    mbar_init(doneBar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    tmap_prefetch(&tin);
    tmap_prefetch(&tout);
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(taddr_s)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // B, for the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  // the weights and barriers above read only constant data; the input
  // (written by the previous kernel) and the output are touched only after it
  // -- unless nothing still running touches them (late: wait before exiting)
  if (!late) pdl_late_entry(0);
  const uint32_t tmem = *taddr_s;

  if (warp == 0) {
    // ---- TMA producer (the whole warp runs the loop; one elected lane issues) ----
    int slot = 0, issued = 0;  // raw stage of the next chunk; chunks issued
    uint32_t ph = 0;           // parity of the stage's current use
    bool ok = true;
    for (long long it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
      int band, s0, T, nch;
      item_geom(a, it, band, s0, T, nch);
      for (int c = 0; c < nch; c++) {
        if (issued >= a.nraw) ok = __all_sync(0xffffffffu, mbar_wait(rawEmpty + 8 * slot, ph ^ 1u));
        if (!ok) {
          if (lane == 0) atomicExch(err, 1);
          break;
        }
        const int p = s0 - r + kPos * c;  // first input position of the chunk
        tma_load_2d_elect(base + L.raw + (uint32_t)(slot * a.rawStride), &tin, p - a.delta, kLines * band,
                          rawFull + 8 * slot, (uint32_t)kRawBytes);
        issued++;
        if (++slot == a.nraw) {
          slot = 0;
          ph ^= 1u;
        }
      }
    }
    // the last load of every stage has landed before the CTA can exit
    for (int k = 0; k < std::min(issued, a.nraw); k++) {
      if (--slot < 0) {
        slot = a.nraw - 1;
        ph ^= 1u;
      }
      if (!mbar_wait(rawFull + 8 * slot, ph) && lane == 0) atomicExch(err, 1);
    }
    __syncwarp();
  } else if (warp <= kConvWarps) {
    // ---- converters: raw chunk -> f16 ring in tensor memory ----
    const int cg = (warp - 1) >> 2;  // converter group: chunks g with g % 2 == cg
    const int q = warp & 3;          // this warp's TMEM lane quarter
    const int m = 32 * q + lane, j = m >> 2, ch = m & 3;
    const uint32_t sel = (uint32_t)ch | ((uint32_t)(ch + 4) << 8);
    const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)kRingCol0;
    int s = 0, seg = 0, n = 0;  // raw stage and ring chunk of chunk n (counted over all chunks)
    uint32_t phs = 0, phr = 0;  // their parities
    bool ok = true;
    for (long long it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
      int band, s0, T, nch;
      item_geom(a, it, band, s0, T, nch);
      for (int c = 0; c < nch; c++) {
        const bool mine = (n & 1) == cg;
        const int cs = s, cseg = seg;
        const uint32_t cphs = phs, cphr = phr;
        const bool reuse = n >= a.nring;
        const int cn = n;
        n++;
        if (++s == a.nraw) {
          s = 0;
          phs ^= 1u;
        }
        if (++seg == a.nring) {
          seg = 0;
          phr ^= 1u;
        }
        if (!mine) continue;
        const bool tr = trace && blockIdx.x == 0 && lane == 0 && q == 1 && cn < kTraceChunks;
        if (tr) g_ring_trace[cg][cn][0] = clock64();
        ok = __all_sync(0xffffffffu, mbar_wait(rawFull + 8 * cs, cphs));
        if (ok && reuse) ok = __all_sync(0xffffffffu, mbar_wait(ringEmpty + 8 * cseg, cphr ^ 1u));
        if (!ok) {
          if (lane == 0) atomicExch(err, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (tr) g_ring_trace[cg][cn][1] = clock64();
        const uint32_t row = base + L.raw + (uint32_t)(cs * a.rawStride + j * (kRawW * 4));
        const int p0 = s0 - r + kPos * c;
        const bool edge = p0 < 0 || p0 + kPos > a.alen;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          // positions 32 h .. 32 h + 31 of the chunk: pixels delta + 32 h + t of the row
          uint32_t qv[36];
#pragma unroll
          for (int v = 0; v < 9; v++) {
            const uint4 d = lds128(row + (uint32_t)(128 * h + 16 * v));
            qv[4 * v] = d.x;
            qv[4 * v + 1] = d.y;
            qv[4 * v + 2] = d.z;
            qv[4 * v + 3] = d.w;
          }
          uint32_t px[32];
#pragma unroll
          for (int t = 0; t < 32; t++) px[t] = qv[t + DELTA];
          if (edge) {
#pragma unroll
            for (int t = 0; t < 32; t++) {
              const int pp = p0 + 32 * h + t;
              if (pp < 0 || pp >= a.alen) px[t] = a.oob;
            }
          }
          uint32_t hv[16];
#pragma unroll
          for (int t = 0; t < 16; t++) hv[t] = sub_pair(px[2 * t], px[2 * t + 1], sel);
          tmem_st16(tq + (uint32_t)(32 * cseg + 16 * h), hv);
        }
        // every lane's tensor-memory stores (and shared-memory reads) are
        // done before the warp's one arrival on each barrier
        asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
        if (tr) g_ring_trace[cg][cn][2] = clock64();
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(rawEmpty + 8 * cs);
          mbar_arrive(ringFull + 8 * cseg);
        }
      }
    }
  } else if (warp == kMmaWarp) {
    // ---- MMA issuer ----
    const uint32_t idesc = instr_desc(128, SPLIT ? 2 * kPos : kPos);
    const uint64_t bdh = mat_desc_sw128(base + L.bhi, 1024);
    constexpr int kBlkShift = SPLIT ? 10 : 9;  // a K block of B is 16 KB (split) or 8 KB, in 16-byte units
    const int kn = a.kspan / 16;                 // K steps of a tile
    const uint32_t ringA = tmem + (uint32_t)kRingCol0;
    int wseg = 0, tseg = 0, acc = 0, tiles = 0;  // next chunk to wait for, the tile's first chunk, accumulator
    uint32_t wph = 0, aph = 0;
    bool ok = true;
    for (long long it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
      int band, s0, T, nch;
      item_geom(a, it, band, s0, T, nch);
      int waited = 0;  // chunks of this item waited for
      for (int i = 0; i < T; i++) {
        const int need = (kPos * i + a.kspan + kPos - 1) / kPos;
        for (; ok && waited < need; waited++) {
          ok = __all_sync(0xffffffffu, mbar_wait(ringFull + 8 * wseg, wph));
          if (++wseg == a.nring) {
            wseg = 0;
            wph ^= 1u;
          }
        }
        if (ok && tiles >= kAcc) ok = __all_sync(0xffffffffu, mbar_wait(tEmpty + 8 * acc, aph ^ 1u));
        if (!ok) {
          if (lane == 0) atomicExch(err, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(acc * accCols);
        // K steps before the ring wraps, then from the ring's start
        const int kw = min(kn, 4 * (a.nring - tseg));
        const uint32_t a0 = ringA + (uint32_t)(32 * tseg);
#pragma unroll 4
        for (int ks = 0; ks < kw; ks++) {
          const uint64_t bo = (uint64_t)(((ks >> 2) << kBlkShift) + ((ks & 3) << 1));  // (block, 32-byte step) >> 4
          mma_ts_elect(d, a0 + 8u * ks, bdh + bo, idesc, ks > 0);
        }
#pragma unroll 4
        for (int ks = kw; ks < kn; ks++) {
          const uint64_t bo = (uint64_t)(((ks >> 2) << kBlkShift) + ((ks & 3) << 1));
          mma_ts_elect(d, ringA + 8u * (ks - kw), bdh + bo, idesc, 1);
        }
        mma_commit_elect(tFull + 8 * acc);
        mma_commit_elect(ringEmpty + 8 * tseg);
        tiles++;
        if (++acc == kAcc) {
          acc = 0;
          aph ^= 1u;
        }
        if (++tseg == a.nring) tseg = 0;
      }
      if (!ok) break;
      for (int c = T; c < nch; c++) {  // the item's halo chunks are read no more
        mma_commit_elect(ringEmpty + 8 * tseg);
        if (++tseg == a.nring) tseg = 0;
      }
    }
    // every issued MMA has finished before tensor memory is freed
    mma_commit_elect(doneBar);
    if (!__all_sync(0xffffffffu, mbar_wait(doneBar, 0)) && lane == 0) atomicExch(err, 1);
    __syncwarp();
  } else {
    // ---- epilogue: two groups of four warps on alternate tiles ----
    const int e = (warp - kEpiWarp0) >> 2;
    const int q = warp & 3;  // TMEM lane quarter of this warp
    const int m = 32 * q + lane, j = m >> 2, ch = m & 3;
    // quad transpose: exchange 16-bit halves with lane ^ 2, then bytes with lane ^ 1
    const uint32_t selA = ch < 2 ? 0x5410u : 0x3276u;
    const uint32_t selB = (ch & 1) ? 0x3715u : 0x6240u;
    const uint64_t k256 = f32x2_splat(256.0f), kq = f32x2_splat(kQuotC24), km = f32x2_splat(kMagic);
    int u = 0, acc = 0;  // tiles seen, their accumulator
    uint32_t aph = 0;
    int mineCount = 0;  // this group's tiles so far (its staging buffer alternates)
    // the group's first warp issues its TMA stores
    const bool issuer = warp == kEpiWarp0 + 4 * e && lane == 0;
    // this lane's line in the staged tile: 16-byte unit (line >> 2) of a
    // 128-byte row, swizzled by the row (position) index mod 8
    const uint32_t unit = (uint32_t)(j >> 2), inUnit = (uint32_t)(j & 3) * 4u;
    bool ok = true;
    for (long long it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
      int band, s0, T, nch;
      item_geom(a, it, band, s0, T, nch);
      for (int i = 0; i < T; i++) {
        const bool mine = (u & 1) == e;
        const int cacc = acc;
        const uint32_t caph = aph;
        u++;
        if (++acc == kAcc) {
          acc = 0;
          aph ^= 1u;
        }
        if (!mine) continue;
        const bool ready = mbar_wait(tFull + 8 * cacc, caph);
        if (!ready && lane == 0) atomicExch(err, 1);
        // the staging buffer of this tile was last read by the store two of
        // the group's tiles back
        if (issuer) bulk_wait_read<1>();
        if (epi_bar_or(e, !ready)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(cacc * accCols);
        const int o0 = s0 + kPos * i;
        const uint32_t stage = base + L.stage + (uint32_t)(2 * e + (mineCount & 1)) * kStageBytes;
        mineCount++;
#pragma unroll
        for (int cc = 0; cc < kPos; cc += 32) {
          float hi[32], lo[32];
          tmem_ld32(ta + (uint32_t)cc, hi);
          if (SPLIT) tmem_ld32(ta + (uint32_t)(kPos + cc), lo);
#pragma unroll
          for (int g4 = 0; g4 < 8; g4++) {
            uint32_t q0, q1, q2, q3;
            const int t = 4 * g4;
            quot2<SPLIT>(hi[t], hi[t + 1], SPLIT ? lo[t] : 0.f, SPLIT ? lo[t + 1] : 0.f, k256, kq, km, q0, q1);
            quot2<SPLIT>(hi[t + 2], hi[t + 3], SPLIT ? lo[t + 2] : 0.f, SPLIT ? lo[t + 3] : 0.f, k256, kq, km, q2,
                         q3);
            // this channel's bytes of positions n .. n + 3, then the quad transpose
            // leaves this lane the whole pixel of position n + ch
            uint32_t w = __byte_perm(__byte_perm(q0, q1, 0x0040u), __byte_perm(q2, q3, 0x0040u), 0x5410u);
            w = __byte_perm(w, __shfl_xor_sync(0xffffffffu, w, 2), selA);
            w = __byte_perm(w, __shfl_xor_sync(0xffffffffu, w, 1), selB);
            const uint32_t row = (uint32_t)(cc + t + ch);  // position within the tile
            asm volatile("st.shared.u32 [%0], %1;\n" ::"r"(stage + row * 128u + (((unit ^ (row & 7u)) << 4) | inUnit)),
                         "r"(w)
                         : "memory");
          }
        }
        // the accumulator is free once its loads are done; the staged tile
        // goes out as one TMA store (rows past the image and lines past the
        // band's end are clipped by the tensor map)
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(tEmpty + 8 * cacc);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        epi_bar(e);
        if (issuer) {
          tma_store_2d(&tout, kLines * band, o0, stage);
          bulk_commit();
        }
      }
    }
    if (issuer) bulk_wait_all();  // the stores have read shared memory and reached global memory
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols)
                 : "memory");
  pdl_late_exit(late);
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

// Row-major image of W x H pixels (u32) with rows pitch pixels apart, boxes
// of bx x by pixels.
bool encode_map(CUtensorMap* m, const void* ptr, int W, int H, long long pitch, int bx, int by,
                bool swizzle128 = false) {
  if (!g_encode) return false;
  cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * 4};
  cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  cuuint32_t estr[2] = {1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// One pass over rows of length alen, clen rows.
bool plan_pass(RingArgs& a, int alen, int clen, int r, int nsm, size_t maxSmem, bool split, int& grid) {
  a.alen = alen;
  a.clen = clen;
  a.opitch = clen;
  a.r = r;
  a.kspan = (kPos + 2 * r + 15) / 16 * 16;
  // the ring takes every TMEM column above the accumulators: the converters run
  // up to (nring - span) chunks ahead of the tile the MMAs read
  a.nring = (kTmemCols - kRingCol0) / 32;
  if (a.nring > kMaxRing || (a.kspan + kPos - 1) / kPos + 1 > a.nring) return false;
  a.delta = (4 - (r & 3)) & 3;  // (s0 - r) mod 4; every s0 is a multiple of 64
  a.rawStride = (kRawBytes + 1023) / 1024 * 1024;
  // as many raw stages as shared memory allows
  a.nraw = kMaxRaw;
  while (a.nraw > 2 && ring_smem(a, split).total + 1024 > maxSmem) a.nraw--;
  if (ring_smem(a, split).total + 1024 > maxSmem) return false;
  // segment length: fewest rounds x (outputs + a fixed cost per item) per
  // CTA.  An item's start (its halo chunks and the hand-offs before its first
  // tile) costs about one tile of 64 outputs at r = 16 and at r = 64
  // (measured on 4096 x 4096: segments of 512 outputs over all SMs beat one
  // whole 4096-pixel row per CTA on 128 SMs by 6 %, and segments of 256 lost
  // it again)
  const long long nband = (clen + kLines - 1) / kLines;
  double best = 1e300;
  for (int T = 1; T <= 64; T++) {
    const int seglen = kPos * T;
    const long long nseg = (alen + seglen - 1) / seglen;
    const long long items = nband * nseg;
    const long long g = std::min<long long>(items, nsm);
    const long long rounds = (items + g - 1) / g;
    const double cost = (double)rounds * (seglen + kPos);
    if (cost < best * 0.999) {
      best = cost;
      a.seglen = seglen;
      a.nseg = (int)nseg;
      a.nitems = items;
      grid = (int)g;
    }
    if (nseg == 1) break;
  }
  return true;
}

template <bool SPLIT>
void launch_ring_pass(const RingArgs& a, int grid, const CUtensorMap& tin, const CUtensorMap& tout,
                      const uint16_t* kern, int* err, int late, cudaStream_t st) {
  // at least 120 KB, so that no second CTA (and tensor-memory allocation) shares an SM
  const size_t smem = std::max<size_t>(ring_smem(a, SPLIT).total + 1024, 120 * 1024);
  switch (a.delta) {
    case 0: launch_pdl(k_blur_ring<SPLIT, 0>, dim3(grid), dim3(kRingThreads), smem, st, tin, tout, a, kern, err, late); break;
    case 1: launch_pdl(k_blur_ring<SPLIT, 1>, dim3(grid), dim3(kRingThreads), smem, st, tin, tout, a, kern, err, late); break;
    case 2: launch_pdl(k_blur_ring<SPLIT, 2>, dim3(grid), dim3(kRingThreads), smem, st, tin, tout, a, kern, err, late); break;
    default: launch_pdl(k_blur_ring<SPLIT, 3>, dim3(grid), dim3(kRingThreads), smem, st, tin, tout, a, kern, err, late); break;
  }
  note_launch();
}

}  // namespace

// True when every weight is an exact f16 (one MMA per K step instead of two).
bool weights_exact_f16(const uint16_t* hostKern, int r) {
  for (int t = 0; t <= 2 * r; t++) {
    uint32_t v = hostKern[t];
    // f16 holds integers of at most 11 significant bits
    while (v >= 2048) {
      if (v & 1) return false;
      v >>= 1;
    }
  }
  return true;
}

// Opt-in shared memory for the ring kernels and the driver's tensor-map
// encoder; false if either is unavailable.
bool ring_blur_init(size_t* maxSmem) {
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return false;
  }
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const void* ks[8] = {(const void*)k_blur_ring<true, 0>,  (const void*)k_blur_ring<true, 1>,
                       (const void*)k_blur_ring<true, 2>,  (const void*)k_blur_ring<true, 3>,
                       (const void*)k_blur_ring<false, 0>, (const void*)k_blur_ring<false, 1>,
                       (const void*)k_blur_ring<false, 2>, (const void*)k_blur_ring<false, 3>};
  for (const void* k : ks)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  *maxSmem = (size_t)optin;
  return true;
}

// Row pitch (pixels) of the transposed intermediate of a blur of an image H
// pixels high: H, or H + 4 when H * 4 bytes is a multiple of 1 KB.  Pass 1
// writes four intermediate rows per warp store and its loads and pass 2's
// read 32 rows per box; at a pitch of a multiple of 1 KB (4096-pixel rows:
// 16 KB) those rows fall on the same memory channels and a 4096 x 4096 blur
// ran 25 % slower than a 4096 x 4100 one.  16 more bytes per row spread them.
long long ring_tmp_pitch(long long H) { return (H * 4) % 1024 == 0 ? H + 4 : H; }

// Bytes of the intermediate buffer a blur of W x H pixels needs.
long long blur_scratch_bytes(long long W, long long H) { return W * ring_tmp_pitch(H) * 4; }

// Both passes (img -> tmp transposed -> img) on the ring kernels.  Returns
// false (and launches nothing) when the image or radius is not for this path:
// width and height must be multiples of 4 (TMA rows of whole 16-byte units
// in both orientations) and both buffers 16-byte aligned, r in 1..128.  tmp
// holds blur_scratch_bytes(W, H) bytes (W rows of ring_tmp_pitch(H) pixels).
bool launch_blur_ring(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                      bool exactF16, uint32_t oob, int nsm, size_t maxSmem, int* err, cudaStream_t st) {
  if (!g_encode || r < 1 || r > 128 || W < 4 || H < 4 || (W & 3) != 0 || (H & 3) != 0 || W > (1 << 24) ||
      H > (1 << 24))
    return false;
  if ((reinterpret_cast<uintptr_t>(img) & 15) || (reinterpret_cast<uintptr_t>(tmp) & 15)) return false;
  // plans and tensor maps of the last few (buffers, size, radius, colour)
  // keys, so a repeated blur costs its two launches on the host (callers
  // hold the library lock)
  struct Plan {
    uint32_t *img, *tmp;
    long long W, H;
    int r, nsm;
    uint32_t oob;
    bool split;
    RingArgs a1, a2;
    int g1, g2;
    CUtensorMap m1, m2;    // pass inputs: image rows, intermediate rows
    CUtensorMap o1, o2;    // pass outputs: intermediate, image (boxes of 32 lines x 64 positions)
  };
  static Plan cache[8];
  static int ncache = 0, next = 0;
  const bool split = !exactF16;
  const Plan* pl = nullptr;
  for (int k = 0; k < ncache; k++) {
    const Plan& c = cache[k];
    if (c.img == img && c.tmp == tmp && c.W == W && c.H == H && c.r == r && c.nsm == nsm && c.oob == oob &&
        c.split == split) {
      pl = &c;
      break;
    }
  }
  if (!pl) {
    Plan n{};
    n.img = img;
    n.tmp = tmp;
    n.W = W;
    n.H = H;
    n.r = r;
    n.nsm = nsm;
    n.oob = oob;
    n.split = split;
    if (!plan_pass(n.a1, (int)W, (int)H, r, nsm, maxSmem, split, n.g1) ||
        !plan_pass(n.a2, (int)H, (int)W, r, nsm, maxSmem, split, n.g2))
      return false;
    n.a1.oob = n.a2.oob = oob;
    n.a1.opitch = (int)ring_tmp_pitch(H);  // pass 1 writes the intermediate
    if (!encode_map(&n.m1, img, (int)W, (int)H, W, kRawW, kLines) ||
        !encode_map(&n.m2, tmp, (int)H, (int)W, ring_tmp_pitch(H), kRawW, kLines) ||
        !encode_map(&n.o1, tmp, (int)H, (int)W, ring_tmp_pitch(H), kLines, kPos, true) ||
        !encode_map(&n.o2, img, (int)W, (int)H, W, kLines, kPos, true))
      return false;
    cache[next] = n;
    pl = &cache[next];
    next = (next + 1) % 8;
    if (ncache < 8) ncache++;
  }
  const Span im{img, (size_t)(W * H * 4)}, tm{tmp, (size_t)blur_scratch_bytes(W, H)};
  const int late1 = dep_late(st, {tm}, {im});  // pass 1: image rows -> intermediate
  if (split)
    launch_ring_pass<true>(pl->a1, pl->g1, pl->m1, pl->o1, kern, err, late1, st);
  else
    launch_ring_pass<false>(pl->a1, pl->g1, pl->m1, pl->o1, kern, err, late1, st);
  const int late2 = dep_late(st, {im}, {tm});  // pass 2 (always waits: it reads pass 1's output)
  if (split)
    launch_ring_pass<true>(pl->a2, pl->g2, pl->m2, pl->o2, kern, err, late2, st);
  else
    launch_ring_pass<false>(pl->a2, pl->g2, pl->m2, pl->o2, kern, err, late2, st);
  return true;
}

// The converter trace: enable != 0 switches it on for later passes (0 off);
// out (if not null) receives up to n values of the last traced pass, laid out
// [group 0..1][chunk 0..255][event 0..2] (0 where nothing was recorded).
int ring_trace(int enable, long long* out, long long n) {
  const int on = enable != 0;
  if (cudaMemcpyToSymbol(g_ring_trace_on, &on, sizeof(int)) != cudaSuccess) return 1;
  if (on) {
    static const long long zero[2 * kTraceChunks * 3] = {};
    if (cudaMemcpyToSymbol(g_ring_trace, zero, sizeof(zero)) != cudaSuccess) return 1;
  }
  if (out && n > 0) {
    const long long cnt = std::min<long long>(n, 2 * kTraceChunks * 3);
    if (cudaMemcpyFromSymbol(out, g_ring_trace, (size_t)cnt * sizeof(long long)) != cudaSuccess) return 1;
  }
  return 0;
}

}  // namespace pxg
