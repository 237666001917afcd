// Gaussian blur passes on the 5th-generation tensor cores (tcgen05, TMEM).
//
// One pass of pixie's blur (images.nim:304-365) is, for every channel,
//   out[x] = (sum_t w[t] * p[x - r + t]) div 256 div 255,   t = 0 .. 2r
// with 8-bit pixels p and 16-bit weights w.  Over a tile of N outputs and the
// K = N + 2r inputs they read, that is a product with a banded (Toeplitz)
// matrix B[n][k] = w[k - n]:  D[m][n] = sum_k A[m][k] * B[n][k], where a row m
// of A is one channel of one image row (X pass) or column (Y pass).
//
// The arithmetic is exact.  Each weight is split into bytes, w = 256 * wh +
// wl, so A (pixels, <= 255) and both weight matrices hold integers <= 255,
// exact in f16; every product is an integer <= 65025 and every sum an integer
// below 2^24 (at most 2r + 1 <= 257 products), exact in the f32 accumulator.
// The epilogue forms 256 * D_hi + D_lo in integers and divides by 65280 --
// bit for bit the reference's integer sums (tests compare every byte with
// the oracle).
//
// Layout: one or two CTAs (256 threads) per SM, persistent over tiles.
// Shared memory holds B_hi and B_lo (built once per CTA) and the A tile, all
// K-major without swizzle: 8 x 8 f16 core matrices of 128 contiguous bytes,
// adjacent in K 128 bytes apart (LBO), adjacent in M/N (K / 8) * 128 bytes
// apart (SBO).  Each tile: the threads convert the tile's pixels to f16 into
// A; one thread issues K/16 MMAs of 128 x N x 16 for each weight byte into
// two TMEM accumulators (N columns each); tcgen05.commit signals an mbarrier;
// the warps read their TMEM lanes back (tcgen05.ld), combine, quantise and
// stage the tile in shared memory for coalesced stores.  Every wait is
// bounded; a wait that runs out sets *err, and the CTA still frees its TMEM.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pxg_device.cuh"
#include "tc_ptx.cuh"

namespace pxg {

void note_launch();

namespace {

using namespace tc;

constexpr int kTcThreads = 256;          // two warpgroups: warps w and w + 4 share TMEM lanes 32 * (w % 4)
}  // namespace

// One pass.  XPASS: rows of A are (image row, channel) pairs, 32 image rows
// per tile, K runs along x; else (image column, channel), 32 columns per
// tile, K along y.  N outputs per tile along the pass axis.
template <bool XPASS, int N>
__global__ void __launch_bounds__(kTcThreads, 2)
    k_blur_tc(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, long long W, long long H, int r,
              int K, const uint16_t* __restrict__ kern, uint32_t oob, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bBytes = (uint32_t)N * K * 2, aBytes = 128u * K * 2;
  unsigned char* bhi = sm;
  unsigned char* blo = sm + bBytes;
  unsigned char* abuf = sm + 2 * bBytes;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(abuf + aBytes);
  uint32_t* taddr_s = reinterpret_cast<uint32_t*>(mbar + 1);

  // The Toeplitz weight bytes, once per CTA.
  for (int i = tid; i < N * K; i += kTcThreads) {
    const int n = i / K, k = i - n * K, t = k - n;
    const uint32_t w = (t >= 0 && t <= 2 * r) ? kern[t] : 0u;
    *reinterpret_cast<uint16_t*>(bhi + canon_off(n, k, K)) = f16_bits(w >> 8);
    *reinterpret_cast<uint16_t*>(blo + canon_off(n, k, K)) = f16_bits(w & 255u);
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {  // 2N TMEM columns: D_hi then D_lo
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(taddr_s)),
                 "r"(2 * N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *taddr_s;
  const uint32_t idesc = instr_desc(128, N);
  const uint32_t sbo = (uint32_t)(K >> 3) * 128u;

  const long long alen = XPASS ? W : H;     // along the pass
  const long long clen = XPASS ? H : W;     // across it
  const long long ntA = (alen + N - 1) / N, ntC = (clen + 31) / 32;
  uint32_t phase = 0;
  bool ok = true;
  for (long long tile = blockIdx.x; tile < ntA * ntC && ok; tile += gridDim.x) {
    const long long a0 = (tile % ntA) * N, c0 = (tile / ntA) * 32;
    // A tile: row m = 4 * j + channel for the j-th line across, K inputs
    // along.  An item is 8 consecutive inputs of one line: 8 loads in flight,
    // then one 16-byte store (a core-matrix row) per channel.
    const int KG = K >> 3;
    for (int it = tid; it < 32 * KG; it += kTcThreads) {
      int j, kg;
      if (XPASS) {  // consecutive threads: consecutive 8-pixel runs of one row
        j = it / KG;
        kg = it - j * KG;
      } else {  // consecutive threads: consecutive columns j
        kg = it >> 5;
        j = it & 31;
      }
      const long long gc = c0 + j;
      uint32_t px[8];
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const long long ga = a0 - r + 8 * kg + t;
        px[t] = 0u;
        if (gc < clen) {
          if (ga >= 0 && ga < alen) px[t] = XPASS ? in[gc * W + ga] : in[ga * W + gc];
          else px[t] = oob;
        }
      }
#pragma unroll
      for (int c = 0; c < 4; c++) {
        uint32_t h[4];
#pragma unroll
        for (int t = 0; t < 4; t++) h[t] = f16_pair(px[2 * t], px[2 * t + 1], c);
        *reinterpret_cast<uint4*>(abuf + canon_off(4 * j + c, 8 * kg, K)) = make_uint4(h[0], h[1], h[2], h[3]);
      }
    }
    // the generic-proxy stores must be visible to the tensor core's reads
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (tid == 0) {
      const uint32_t a = smem_u32(abuf), bh = smem_u32(bhi), bl = smem_u32(blo);
      for (int s = 0; s < K / 16; s++) {
        const uint32_t off = (uint32_t)s * 256u;  // two core matrices along K per step
        mma_f16(tmem, mat_desc(a + off, 128, sbo), mat_desc(bh + off, 128, sbo), idesc, s > 0);
        mma_f16(tmem + N, mat_desc(a + off, 128, sbo), mat_desc(bl + off, 128, sbo), idesc, s > 0);
      }
      mma_commit(smem_u32(mbar));
    }
    const bool waited = mbar_wait(smem_u32(mbar), phase);
    if (!waited && lane == 0) atomicExch(err, 1);
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (__syncthreads_or(!waited)) {  // every thread leaves together, then frees TMEM below
      ok = false;
      break;
    }
    // epilogue: warp w reads TMEM lanes m = 32 * (w % 4) + lane, columns
    // [(w / 4) * N / 2, + N / 2); the tile is staged as bytes [j][n][c] with a
    // row stride of 4 * N + 16 bytes (quads of lanes land in different banks)
    const int q = warp & 3, half = warp >> 2;
    const int m = 32 * q + lane, j = m >> 2, c = m & 3;
    unsigned char* stage = abuf;  // the A tile is no longer read
    const int rs = 4 * N + 16;
#pragma unroll 1
    for (int cc = half * (N / 2); cc < (half + 1) * (N / 2); cc += 32) {
      float hi[32], lo[32];
      tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)cc, hi);
      tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(N + cc), lo);
#pragma unroll
      for (int t = 0; t < 32; t++) {
        const uint32_t v = (uint32_t)hi[t] * 256u + (uint32_t)lo[t];
        stage[j * rs + (cc + t) * 4 + c] = (unsigned char)(v / 65280u);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    const uint32_t* st = reinterpret_cast<const uint32_t*>(stage);
    for (int i = tid; i < 32 * N; i += kTcThreads) {
      int jj, n;
      if (XPASS) {  // a row's N outputs are contiguous
        jj = i / N;
        n = i - jj * N;
      } else {  // 32 columns of one output row are contiguous
        n = i >> 5;
        jj = i & 31;
      }
      const long long ga = a0 + n, gc = c0 + jj;
      if (ga < alen && gc < clen) {
        const uint32_t v = st[jj * (rs / 4) + n];
        if (XPASS) out[gc * W + ga] = v;
        else out[ga * W + gc] = v;
      }
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * N) : "memory");
}

// The pipelined pass: warp-specialised, with S (2..4) input slots, so that loading
// and converting tile i + 1, the MMAs of tile i and the epilogue of tile i - 1
// run at the same time.
//   warps 0-7   producers (two groups taking alternate tiles): global loads
//               -> f16 A tile in A[i % S], then arrive on full[i % S];
//               before refilling a slot they wait empty[slot]
//   warp 16     one thread issues the MMAs of a tile into accumulator pair
//               i % 4 (TMEM) and commits to empty[slot] and tfull[pair]
//   warps 8-15  epilogue, two groups of four warps on alternate tiles: wait
//               tfull[pair], read TMEM lanes 32 * (w % 4), arrive on
//               tempty[pair], quantise, stage and store the tile
// Every mbarrier wait is bounded; a role whose wait runs out sets *err and
// stops, the others' waits then run out too, and the CTA frees its TMEM.
constexpr int kPipeThreads = 544;  // 8 producer warps, 8 epilogue warps, 1 MMA warp
constexpr int kProducers = 256, kEpilogue = 256;

template <bool XPASS, int N>
__global__ void __launch_bounds__(kPipeThreads, 1)
    k_blur_tcp(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, long long W, long long H, int r,
               int K, int S, const uint16_t* __restrict__ kern, uint32_t oob, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bBytes = (uint32_t)N * K * 2, aBytes = 128u * K * 2;
  const int rs = 4 * N + 16;  // output staging row stride (bytes)
  unsigned char* bhi = sm;
  unsigned char* blo = sm + bBytes;
  unsigned char* abuf0 = sm + 2 * bBytes;  // S input slots
  unsigned char* stage = abuf0 + (size_t)S * aBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(stage + 2 * 32 * rs);  // full[4] empty[4] tfull[4] tempty[4]
  uint32_t* taddr_s = reinterpret_cast<uint32_t*>(bars + 16);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + 4), tfull0 = smem_u32(bars + 8),
                 tempty0 = smem_u32(bars + 12);

  for (int i = tid; i < N * K; i += kPipeThreads) {
    const int n = i / K, k = i - n * K, t = k - n;
    const uint32_t w = (t >= 0 && t <= 2 * r) ? kern[t] : 0u;
    *reinterpret_cast<uint16_t*>(bhi + canon_off(n, k, K)) = f16_bits(w >> 8);
    *reinterpret_cast<uint16_t*>(blo + canon_off(n, k, K)) = f16_bits(w & 255u);
  }
  if (tid == 0) {
    for (int b = 0; b < 4; b++) {
      mbar_init(full0 + 8 * b, kProducers / 2);
      mbar_init(empty0 + 8 * b, 1);
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, kEpilogue / 2);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {  // four accumulator pairs: (D_hi, D_lo) x 4
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(taddr_s)),
                 "r"(8 * N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // B, for the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *taddr_s;

  const long long alen = XPASS ? W : H, clen = XPASS ? H : W;
  const long long ntA = (alen + N - 1) / N, ntC = (clen + 31) / 32, ntiles = ntA * ntC;
  const long long nmine = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  if (tid < kProducers) {
    // producers, in two groups of 128 threads taking alternate tiles, so two
    // tiles' loads are in flight at once
    const int KG = K >> 3;
    const int grp = tid >> 7, gtid = tid & 127;
    // 16-byte loads along x when every run of 8 starts on a 16-byte boundary
    const bool vec = XPASS && (W & 3) == 0 && (r & 3) == 0 &&
                     ((reinterpret_cast<uintptr_t>(in) & 15) == 0);
    for (long long i = grp; i < nmine; i += 2) {
      const int slot = (int)(i % S);
      if (i >= S && !mbar_wait(empty0 + 8 * slot, (uint32_t)((i / S - 1) & 1))) {
        if (lane == 0) atomicExch(err, 1);
        break;
      }
      const long long tile = blockIdx.x + i * gridDim.x;
      const long long a0 = (tile % ntA) * N, c0 = (tile / ntA) * 32;
      unsigned char* abuf = abuf0 + slot * aBytes;
      // two items per round: 16 pixels' loads in flight before any is converted
      for (int it0 = gtid; it0 < 32 * KG; it0 += 256) {
        uint32_t px[2][8];
        int jj[2], kk[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const int it = it0 + 128 * u;
          int j = 0, kg = 0;
          if (XPASS) {
            j = it / KG;
            kg = it - j * KG;
          } else {
            kg = it >> 5;
            j = it & 31;
          }
          jj[u] = j;
          kk[u] = kg;
          const long long gc = c0 + j, g0 = a0 - r + 8 * kg;
          const bool live = it < 32 * KG && gc < clen;
          if (XPASS && live && vec && g0 >= 0 && g0 + 8 <= alen) {
            // the run's 8 pixels as two aligned 16-byte loads
            const uint4 v0 = *reinterpret_cast<const uint4*>(in + gc * W + g0);
            const uint4 v1 = *reinterpret_cast<const uint4*>(in + gc * W + g0 + 4);
            px[u][0] = v0.x; px[u][1] = v0.y; px[u][2] = v0.z; px[u][3] = v0.w;
            px[u][4] = v1.x; px[u][5] = v1.y; px[u][6] = v1.z; px[u][7] = v1.w;
          } else {
#pragma unroll
            for (int t = 0; t < 8; t++) {
              const long long ga = g0 + t;
              px[u][t] = 0u;
              if (live) {
                if (ga >= 0 && ga < alen) px[u][t] = XPASS ? in[gc * W + ga] : in[ga * W + gc];
                else px[u][t] = oob;
              }
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
          if (it0 + 128 * u >= 32 * KG) break;
#pragma unroll
          for (int c = 0; c < 4; c++) {
            uint32_t h[4];
#pragma unroll
            for (int t = 0; t < 4; t++) h[t] = f16_pair(px[u][2 * t], px[u][2 * t + 1], c);
            *reinterpret_cast<uint4*>(abuf + canon_off(4 * jj[u] + c, 8 * kk[u], K)) =
                make_uint4(h[0], h[1], h[2], h[3]);
          }
        }
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      mbar_arrive(full0 + 8 * slot);
    }
  } else if (warp == 16) {
    // the MMA issuer
    if (lane == 0) {
      const uint32_t idesc = instr_desc(128, N);
      const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
      const uint32_t bh = smem_u32(bhi), bl = smem_u32(blo);
      for (long long i = 0; i < nmine; i++) {
        const int slot = (int)(i % S), pair = (int)(i & 3);
        if (!mbar_wait(full0 + 8 * slot, (uint32_t)((i / S) & 1)) ||
            (i >= 4 && !mbar_wait(tempty0 + 8 * pair, (uint32_t)(((i >> 2) - 1) & 1)))) {
          atomicExch(err, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t a = smem_u32(abuf0 + slot * aBytes);
        const uint32_t dh = tmem + (uint32_t)(pair * 2 * N), dl = dh + (uint32_t)N;
        for (int s2 = 0; s2 < K / 16; s2++) {
          const uint32_t off = (uint32_t)s2 * 256u;
          mma_f16(dh, mat_desc(a + off, 128, sbo), mat_desc(bh + off, 128, sbo), idesc, s2 > 0);
          mma_f16(dl, mat_desc(a + off, 128, sbo), mat_desc(bl + off, 128, sbo), idesc, s2 > 0);
        }
        mma_commit(empty0 + 8 * slot);
        mma_commit(tfull0 + 8 * pair);
      }
    }
    __syncwarp();
  } else {
    // epilogue: two groups of four warps (8-11, 12-15) take alternate tiles;
    // in a group, warp w reads TMEM lanes 32 * (w % 4), every column
    const int q = warp & 3, grp = (warp - 8) >> 2;
    const int m = 32 * q + lane, j = m >> 2, c = m & 3;
    const int etid = (tid - kProducers) & 127;
    unsigned char* st8 = stage + grp * 32 * rs;
    for (long long i = grp; i < nmine; i += 2) {
      const int pair = (int)(i & 3);
      const bool ready = mbar_wait(tfull0 + 8 * pair, (uint32_t)((i >> 2) & 1));
      if (!ready && lane == 0) atomicExch(err, 1);
      // also: the group's staging buffer is free (its previous stores are done)
      if (epi_bar_or(grp, !ready)) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t dh = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(pair * 2 * N);
#pragma unroll 1
      for (int cc = 0; cc < N; cc += 32) {
        float hi[32], lo[32];
        tmem_ld32(dh + (uint32_t)cc, hi);
        tmem_ld32(dh + (uint32_t)(N + cc), lo);
#pragma unroll
        for (int t = 0; t < 32; t++) {
          const uint32_t v = (uint32_t)hi[t] * 256u + (uint32_t)lo[t];
          st8[j * rs + (cc + t) * 4 + c] = (unsigned char)(v / 65280u);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      mbar_arrive(tempty0 + 8 * pair);
      epi_bar(grp);
      const long long tile = blockIdx.x + i * gridDim.x;
      const long long a0 = (tile % ntA) * N, c0 = (tile / ntA) * 32;
      const uint32_t* st = reinterpret_cast<const uint32_t*>(st8);
      for (int e = etid; e < 32 * N; e += 128) {
        int jj, n;
        if (XPASS) {
          jj = e / N;
          n = e - jj * N;
        } else {
          n = e >> 5;
          jj = e & 31;
        }
        const long long ga = a0 + n, gc = c0 + jj;
        if (ga < alen && gc < clen) {
          const uint32_t v = st[jj * (rs / 4) + n];
          if (XPASS) out[gc * W + ga] = v;
          else out[ga * W + gc] = v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(8 * N) : "memory");
}

// The pipelined pass's tile width: 64 outputs for r <= 64, 32 up to 128
// (the input slots, B and the output stages fit 227 KB of shared memory).
// Below r = 8 the CUDA-core kernels are as fast or faster (the pass is not
// compute-bound there), and they take those radii.
int tcp_blur_n(int r) { return r < 8 || r > 128 ? 0 : (r <= 64 ? 64 : 32); }
int tcp_blur_k(int r) {
  const int n = tcp_blur_n(r);
  return n ? (n + 2 * r + 15) / 16 * 16 : 0;
}
size_t tcp_blur_smem(int r, int slots) {
  const int n = tcp_blur_n(r), k = tcp_blur_k(r);
  return n ? (size_t)2 * n * k * 2 + (size_t)slots * 128 * k * 2 + (size_t)2 * 32 * (4 * n + 16) + 16 * 8 + 16
           : 0;
}
// Input slots of the pipeline: as many as fit, up to 4.
int tcp_blur_slots(int r, size_t maxSmem) {
  int sl = 4;
  while (sl > 2 && tcp_blur_smem(r, sl) > maxSmem) sl--;
  return sl;
}
const void* tcp_blur_kernel(bool x, int n) {
  if (n == 64) return x ? (const void*)k_blur_tcp<true, 64> : (const void*)k_blur_tcp<false, 64>;
  return x ? (const void*)k_blur_tcp<true, 32> : (const void*)k_blur_tcp<false, 32>;
}

// Tile width along the pass and the padded input span for radius r, or 0 when
// the tensor path does not take r: it keeps every sum below 2^24 for r <= 128,
// and below r = 8 the CUDA-core kernels, which are not compute-bound there,
// are faster.
int tc_blur_n(int r) { return r < 8 || r > 128 ? 0 : (r <= 64 ? 128 : 64); }
int tc_blur_k(int r) {
  const int n = tc_blur_n(r);
  return n ? (n + 2 * r + 15) / 16 * 16 : 0;
}
size_t tc_blur_smem(int r) {
  const int n = tc_blur_n(r), k = tc_blur_k(r);
  return n ? (size_t)2 * n * k * 2 + (size_t)128 * k * 2 + 16 : 0;
}
const void* tc_blur_kernel(bool x, int n) {
  if (n == 128) return x ? (const void*)k_blur_tc<true, 128> : (const void*)k_blur_tc<false, 128>;
  return x ? (const void*)k_blur_tc<true, 64> : (const void*)k_blur_tc<false, 64>;
}

// Both passes with the pipelined kernel.  Returns false if r is not for it.
bool launch_blur_tcp(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                     uint32_t oob, int nsm, size_t maxSmem, int* err, cudaStream_t st) {
  const int n = tcp_blur_n(r), k = tcp_blur_k(r);
  const int slots = tcp_blur_slots(r, maxSmem);
  const size_t smem = tcp_blur_smem(r, slots);
  if (!n || smem > maxSmem) return false;
  const long long tilesX = ((W + n - 1) / n) * ((H + 31) / 32);
  const long long tilesY = ((H + n - 1) / n) * ((W + 31) / 32);
  const unsigned gx = (unsigned)std::max<long long>(1, std::min<long long>(tilesX, nsm));
  const unsigned gy = (unsigned)std::max<long long>(1, std::min<long long>(tilesY, nsm));
  if (n == 64) {
    k_blur_tcp<true, 64><<<gx, kPipeThreads, smem, st>>>(img, tmp, W, H, r, k, slots, kern, oob, err);
    k_blur_tcp<false, 64><<<gy, kPipeThreads, smem, st>>>(tmp, img, W, H, r, k, slots, kern, oob, err);
  } else {
    k_blur_tcp<true, 32><<<gx, kPipeThreads, smem, st>>>(img, tmp, W, H, r, k, slots, kern, oob, err);
    k_blur_tcp<false, 32><<<gy, kPipeThreads, smem, st>>>(tmp, img, W, H, r, k, slots, kern, oob, err);
  }
  note_launch();
  note_launch();
  return true;
}

// Both passes (img -> tmp -> img).  Returns false if r is not for this path.
bool launch_blur_tc(uint32_t* img, uint32_t* tmp, long long W, long long H, int r, const uint16_t* kern,
                    uint32_t oob, int nsm, size_t maxSmem, int* err, cudaStream_t st) {
  const int n = tc_blur_n(r), k = tc_blur_k(r);
  const size_t smem = tc_blur_smem(r);
  if (!n || smem > maxSmem) return false;
  const long long tilesX = ((W + n - 1) / n) * ((H + 31) / 32);
  const long long tilesY = ((H + n - 1) / n) * ((W + 31) / 32);
  // two CTAs per SM when both fit in shared memory (their TMEM, 2 x 2N
  // columns, always fits the SM's 512): one stages while the other computes
  const int per = smem * 2 + 2048 <= 228 * 1024 ? 2 : 1;
  const unsigned gx = (unsigned)std::max<long long>(1, std::min<long long>(tilesX, (long long)nsm * per));
  const unsigned gy = (unsigned)std::max<long long>(1, std::min<long long>(tilesY, (long long)nsm * per));
  if (n == 128) {
    k_blur_tc<true, 128><<<gx, kTcThreads, smem, st>>>(img, tmp, W, H, r, k, kern, oob, err);
    k_blur_tc<false, 128><<<gy, kTcThreads, smem, st>>>(tmp, img, W, H, r, k, kern, oob, err);
  } else {
    k_blur_tc<true, 64><<<gx, kTcThreads, smem, st>>>(img, tmp, W, H, r, k, kern, oob, err);
    k_blur_tc<false, 64><<<gy, kTcThreads, smem, st>>>(tmp, img, W, H, r, k, kern, oob, err);
  }
  note_launch();
  note_launch();
  return true;
}

}  // namespace pxg
