// Tensor-core (tcgen05) Fourier densities over the whole half-space lattice.
//
// rho[(nx,ny), nz] = sum_j W_j(nx,ny) Z_j(nz), W = X(nx) Y(ny), is a complex
// GEMM with the atoms as the reduction axis.  As a real GEMM per tile of 64
// complex (nx,ny) rows (8 nx x 8 ny) and n consecutive nz:
//   A (128 x 2J): lane 2r   = [Wr, -Wi] of complex row r (k = 2j, 2j+1 per atom j)
//                 lane 2r+1 = [Wi,  Wr]
//   B (  n x 2J): [Zr, Zi] for n consecutive nz (n <= 128, a multiple of 16,
//                 sized per tile to the nz extent of its 64 rows)
//   D = A B^T  (128 x n): lane 2r = Re rho, lane 2r + 1 = Im rho.
// The lane pair of a complex row sits in one tensor-memory lane quadrant, so
// one warp writes both rows.  Lane 2r holds conj(X) conj(Y) and lane 2r + 1
// holds (i conj(X)) conj(Y): both are one complex product of a per-lane X
// variant and conj(Y), so the builders need no sign or swap fix-ups.
// Operands are FP16 split into hi + lo parts (hi = x rounded to a multiple of
// 2^-11, exact in FP16; lo = x - hi to ~2^-24), and each chunk of 32 atoms
// runs three tcgen05.mma passes, hi*lo + lo*hi + hi*hi (small terms first),
// accumulating in FP32 tensor memory.  The tensor core's FP32 accumulation
// drops low bits as the accumulator grows, so an accumulation never spans more
// than TC_GROUP chunks (64 atoms): the drain warps then add the accumulator
// into compensated sums held in their registers (Fast2Sum) and write the
// rounding residual back into the accumulator, where the next accumulation on
// it starts.  The phases are the exact fixed-point phases of the FP32 kernels
// (fraction of the box in units of 2^-31 turns).
//
// Per frame batch, zgen_kernel precomputes the B operands (Z hi/lo in the
// K-major 128-byte-swizzled layout, one blob per (frame, nz window, chunk)) and
// xygen_kernel the X and Y phase tables.  The main kernel is warp-specialised,
// one CTA per SM, 512 tensor-memory columns (two 128-column accumulators, four
// 64-column A stages):
//   warps 0-7    drain: accumulator -> register sums (lane quadrant warp % 4,
//                16-column blocks 2 i + warp / 4), then the epilogue
//   warp 8       producer: bulk copies (cp.async.bulk) of Z hi/lo and the X/Y
//                tables of each chunk into a 4-stage shared-memory ring (stages
//                sized to the nz window)
//   warps 9-10   MMA issuers, one per accumulator (alternate 64-atom groups):
//                12 tcgen05.mma per chunk, A read from tensor memory
//   warps 11-18  builders: the A operand of the chunk (W products, FP16 split)
//                stored into tensor memory (lane quadrant warp % 4, atoms
//                16 x ((warp - 11) / 4) onwards)
// Hand-offs are mbarriers (bulk-copy transactions, tcgen05.commit, thread
// arrivals); every wait is bounded, and a timeout makes every role stop, wait
// for its own copies and MMAs, free tensor memory and report through an error
// word.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "f32x2.cuh"
#include "tc_tiles.h"
#include "umma.cuh"

namespace amdat {

constexpr int TC_J = 32;                      // atoms per chunk
constexpr int TC_K = 2 * TC_J;                // real K per chunk
constexpr int TC_ROWS = 64;                   // complex rows (8 nx x 8 ny)
constexpr int TC_NMAX = 128;                  // widest nz window (MMA N)
constexpr int TC_M = 2 * TC_ROWS;             // MMA M = 128
constexpr int TC_GROUP = 2;                   // chunks per tensor-memory accumulation
constexpr int TC_S = 4;                       // ring stages: Z, X, Y in shared memory, A in tensor memory
constexpr uint32_t TC_HDR = 1024;             // barrier header ahead of the ring
constexpr uint32_t TC_SMEM_MAX = 227 * 1024;  // dynamic shared memory per block
constexpr int TC_DRAIN_WARPS = 8;             // warps 0-7
constexpr int TC_DRAIN_PAR = TC_DRAIN_WARPS / 4;  // drain warps per lane quadrant
constexpr int TC_PRODUCER_WARP = 8;
constexpr int TC_MMA_WARP = 9;                // warps 9 and 10: one per accumulator
constexpr int TC_MMA_WARPS = 2;
constexpr int TC_BUILD_WARP0 = TC_MMA_WARP + TC_MMA_WARPS;  // warps 11-18
constexpr int TC_BUILD_WARPS = 8;
constexpr int TC_THREADS = 32 * (TC_BUILD_WARP0 + TC_BUILD_WARPS);  // 608
constexpr uint32_t TC_XB = TC_J * 2 * 8 * sizeof(float2);     // 4 KB: 32 atoms x 2 lane variants x 8 nx
constexpr uint32_t TC_YB = TC_J * 8 * sizeof(float2);         // 2 KB: 32 atoms x 8 ny
constexpr uint32_t TC_XYB = TC_XB + TC_YB;                    // one (block, chunk) table pair
constexpr uint32_t TC_WAIT = 1u << 19;                        // try_wait calls of <= 1 us (~0.5 s bound)
// tensor-memory columns: two accumulators, then four A stages of 64 columns:
// per 16-atom half u, [hi (16 columns) | lo (16 columns)] at 32 u
constexpr uint32_t TC_COL_ACC = 0, TC_COL_A = 2 * TC_NMAX, TC_A_COLS = 2 * (TC_K / 2);
constexpr uint32_t TC_TMEM_COLS = 512;
static_assert(TC_COL_A + TC_S * TC_A_COLS <= TC_TMEM_COLS, "accumulators and A stages must fit tensor memory");

struct TcHdr {
  uint64_t full_z[TC_S];  // the stage's copies landed
  uint64_t full_a[TC_S];  // the stage's A operand built
  uint64_t empty[TC_S];   // the stage's MMAs finished (shared-memory and tensor-memory halves)
  uint64_t full_acc[2], empty_acc[2];
  uint64_t mma_done;
  uint32_t tmem;
  volatile int bad;  // any role gave up
  int z_issued;      // bulk copies issued
};
static_assert(sizeof(TcHdr) <= TC_HDR, "the barrier header must fit its slot");
// the Z operands use the 128-byte-swizzled K-major layout: 128-byte rows, 1024-byte aligned tiles
static_assert(TC_K * 2 == 128, "one chunk's K must fill a 128-byte swizzle row");

// shared-memory ring stage bytes for nz windows of nzw: Z hi, Z lo (nzw rows of
// 128 bytes each, 1024-byte aligned for a multiple of 8 rows), X, Y
__host__ __device__ constexpr uint32_t tc_zstage(int nzw) { return 2u * (uint32_t)nzw * TC_K * 2 + TC_XYB; }

__device__ __forceinline__ void tc_split(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(__fsub_rn(x, __half2float(hi)));
}

__device__ __forceinline__ void tc_phase(int32_t ph, float* s, float* c) {
  sincospif(__fmul_rn((float)ph, 9.313225746154785e-10f), s, c);  // ph * 2^-30 * pi
}

// hi/lo FP16 pair of (a, b) with |a|, |b| <= 1: hi = round to a multiple of
// 2^-11 (6144 = 1.5 * 2^12 has a 2^-11 ulp, so (x + 6144) - 6144 rounds x to
// that grid; every such value in [-1, 1] is exact in FP16), lo = x - hi exactly
// in FP32 (|lo| <= 2^-12), rounded once to FP16.  Packed as (a: low half, b: high half).
__device__ __forceinline__ void tc_split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const uint64_t w = pk2(a, b), c = pk2(6144.0f, 6144.0f);
  const uint64_t h = sub2(add2(w, c), c);
  const uint64_t l = sub2(w, h);
  float ha, hb, la, lb;
  upk2(h, ha, hb);
  upk2(l, la, lb);
  const __half2 H = __floats2half2_rn(ha, hb), L = __floats2half2_rn(la, lb);
  hi = *reinterpret_cast<const uint32_t*>(&H);
  lo = *reinterpret_cast<const uint32_t*>(&L);
}

// Z operands of one frame batch: blob (f, zblk, chunk) = [hi][lo], each an
// nzw (nz) x 64 (k) K-major tile; k = 2j -> Re Z_j, 2j+1 -> Im Z_j
__global__ void __launch_bounds__(256)
    zgen_kernel(const int4* __restrict__ fx, int32_t n_list, int32_t n_chunks, int32_t n_zblk,
                int32_t nzw, unsigned char* __restrict__ zbuf) {
  const int blob = blockIdx.x;
  const int c = blob % n_chunks;
  const int zb = (blob / n_chunks) % n_zblk;
  const int f = blob / (n_chunks * n_zblk);
  const uint32_t half = (uint32_t)nzw * TC_K * 2;
  unsigned char* hi = zbuf + (size_t)blob * 2 * half;
  unsigned char* lo = hi + half;
  const int4* F = fx + (int64_t)f * n_list;
  for (int e = threadIdx.x; e < nzw * TC_J; e += blockDim.x) {
    const int col = e % nzw, j = e / nzw;
    const int a = c * TC_J + j;
    float s = 0.f, co = 0.f;
    if (a < n_list) {
      const int32_t nz = zb * nzw + col;
      tc_phase((int32_t)((uint32_t)nz * (uint32_t)F[a].z), &s, &co);
    }
    __half rh, rl, ih, il;
    tc_split(co, rh, rl);
    tc_split(s, ih, il);
    const uint32_t off = umma::kmajor_sw128_offset(col, 2 * j);
    *reinterpret_cast<__half2*>(hi + off) = __halves2half2(rh, ih);
    *reinterpret_cast<__half2*>(lo + off) = __halves2half2(rl, il);
  }
}

// X and Y phase tables of one frame batch.  For block b of 8 lattice indices
// (n = -nmax + 8 b + m) and chunk c of 32 atoms, TC_XYB bytes at
// (f * n_blk + b) * n_chunks + c; atom pair p = j / 2, element j % 2 of a float4:
//   X (4 KB): float4 p * 16 + m * 2 + v, the lane variant v of
//             X_j(n) = exp(i 2 pi n qx_j): v = 0 conj(X) = (cos, -sin),
//             v = 1 i conj(X) = (sin, cos)
//   Y (2 KB): float4 p * 8 + m, Y_j(n) = (cos, sin)
// The eight lanes of a builder quarter warp (four nx, both variants, one ny)
// read eight distinct bank groups of X and one broadcast float4 of Y.
__global__ void __launch_bounds__(256)
    xygen_kernel(const int4* __restrict__ fx, int32_t n_list, int32_t n_chunks, int32_t n_blk,
                 int32_t nmax, float2* __restrict__ xybuf) {
  const int blk = blockIdx.x;  // (f * n_blk + b) * n_chunks + c
  const int c = blk % n_chunks;
  const int b = (blk / n_chunks) % n_blk;
  const int f = blk / (n_chunks * n_blk);
  float2* X = xybuf + (size_t)blk * (TC_XYB / sizeof(float2));
  float2* Y = X + TC_XB / sizeof(float2);
  const int4* F = fx + (int64_t)f * n_list;
  const int e = threadIdx.x;  // 256 = 32 atoms x 8 indices
  const int j = e >> 3, m = e & 7, p = j >> 1;
  const int a = c * TC_J + j;
  float xs = 0.f, xc = 0.f, ys = 0.f, yc = 0.f;
  if (a < n_list) {
    const int32_t n = -nmax + 8 * b + m;
    tc_phase((int32_t)((uint32_t)n * (uint32_t)F[a].x), &xs, &xc);
    tc_phase((int32_t)((uint32_t)n * (uint32_t)F[a].y), &ys, &yc);
  }
  X[(p * 16 + m * 2 + 0) * 2 + (j & 1)] = make_float2(xc, -xs);
  X[(p * 16 + m * 2 + 1) * 2 + (j & 1)] = make_float2(xs, xc);
  Y[(p * 8 + m) * 2 + (j & 1)] = make_float2(yc, ys);
}

// warp-uniform bounded wait: lane 0 reads the block's error flag and polls,
// the warp shares the outcome (false: give up)
__device__ __forceinline__ bool warp_wait(uint64_t* mbar, uint32_t parity, volatile int* bad) {
  bool ok = true;
  if ((threadIdx.x & 31) == 0) ok = !*bad && umma::mbar_wait(mbar, parity, TC_WAIT);
  return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    rhok_tc_kernel(int32_t n_list, int32_t n_chunks, int32_t n_zblk, int32_t nzw, int32_t n_blk,
                   int32_t nmax, const TcTile* __restrict__ tiles,
                   const int32_t* __restrict__ entry_k, const unsigned char* __restrict__ zbuf,
                   const float2* __restrict__ xybuf, int32_t frame0, int32_t n_k, float2* __restrict__ rho,
                   int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~(uintptr_t)1023);
  TcHdr& S = *reinterpret_cast<TcHdr*>(base);
  unsigned char* ring = base + TC_HDR;  // TC_S stages of zstage bytes
  const TcTile T = tiles[blockIdx.x];
  const int fl = blockIdx.y;  // frame within the batch
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = T.n;
  const uint32_t zhalf = (uint32_t)nzw * TC_K * 2, zstage = tc_zstage(nzw);
  const unsigned char* Z = zbuf + ((size_t)fl * n_zblk + T.zblk) * (size_t)n_chunks * 2 * zhalf;
  constexpr size_t XY_F2 = TC_XYB / sizeof(float2);
  const float2* XT = xybuf + ((size_t)fl * n_blk + (T.nx0 + nmax) / 8) * (size_t)n_chunks * XY_F2;
  const float2* YT = xybuf + ((size_t)fl * n_blk + (T.ny0 + nmax) / 8) * (size_t)n_chunks * XY_F2 +
                     TC_XB / sizeof(float2);
  const int n_groups = (n_chunks + TC_GROUP - 1) / TC_GROUP;

  if (tid == 0) {
    for (int s = 0; s < TC_S; ++s) {
      umma::mbar_init(&S.full_z[s], 1);
      umma::mbar_init(&S.full_a[s], TC_BUILD_WARPS);
      umma::mbar_init(&S.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(&S.full_acc[b], 1);
      umma::mbar_init(&S.empty_acc[b], TC_DRAIN_WARPS);
    }
    umma::mbar_init(&S.mma_done, TC_MMA_WARPS);
    umma::fence_mbarrier_init();
    S.bad = 0;
    S.z_issued = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(&S.tmem, TC_TMEM_COLS);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = S.tmem;
  const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;  // this warp's tensor-memory lane quadrant

  if (warp == TC_PRODUCER_WARP) {
    // ---- producer: Z(c), X(c), Y(c) into ring stage c % TC_S once the MMAs of c - TC_S are done
    if (lane == 0) {
      int c = 0;
      for (; c < n_chunks; ++c) {
        const int s = c % TC_S;
        if (S.bad || !umma::mbar_wait(&S.empty[s], ((c / TC_S) & 1) ^ 1, TC_WAIT)) {
          S.bad = 1;
          break;
        }
        unsigned char* dst = ring + (size_t)s * zstage;
        const unsigned char* src = Z + (size_t)c * 2 * zhalf;
        umma::mbar_expect_tx(&S.full_z[s], 2u * n * TC_K * 2 + TC_XYB);
        umma::bulk_g2s(dst, src, (uint32_t)n * TC_K * 2, &S.full_z[s]);
        umma::bulk_g2s(dst + zhalf, src + zhalf, (uint32_t)n * TC_K * 2, &S.full_z[s]);
        umma::bulk_g2s(dst + 2 * zhalf, XT + (size_t)c * XY_F2, TC_XB, &S.full_z[s]);
        umma::bulk_g2s(dst + 2 * zhalf + TC_XB, YT + (size_t)c * XY_F2, TC_YB, &S.full_z[s]);
      }
      S.z_issued = c;
    }
  } else if (warp >= TC_MMA_WARP && warp < TC_MMA_WARP + TC_MMA_WARPS) {
    // ---- MMA issuers: warp TC_MMA_WARP + b issues the groups of accumulator b
    // (even / odd groups), so two threads keep the tensor pipe fed; the two
    // accumulators are independent, and each chunk is read by one issuer
    const int mine = warp - TC_MMA_WARP;
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_f16_f32(TC_M, n);
      // the B descriptor's address field is the byte address >> 4 (14 bits, all
      // of shared memory), so the ring stage, the lo half (both 1024-byte
      // aligned) and the k-step (32 B inside the swizzled 128-byte rows) add to
      // it; k-step ks (atoms 8 ks .. 8 ks + 7) of the A stage is column
      // 32 (ks / 2) + 8 (ks % 2), its lo part 16 columns on
      const uint64_t b_desc0 = umma::smem_desc_sw128(umma::smem_addr(ring));
      const uint32_t b_stage16 = zstage >> 4, b_lo16 = zhalf >> 4;
      constexpr uint32_t A_LO = 16;
      static_assert(TC_S == 2 * TC_GROUP, "a ring cycle holds one group of each accumulator");
      // the chunk loop is unrolled over the ring, so the stage (sd) and the
      // accumulator (sd / TC_GROUP) of every MMA are offsets from loop-invariant
      // bases: one thread issues a tcgen05.mma in ~50 cycles at best, and
      // per-MMA arithmetic or waits add to that
      bool ok = true;
      for (int c0 = 0; c0 < n_chunks && ok; c0 += TC_S) {
#pragma unroll
        for (int sd = 0; sd < TC_S; ++sd) {
          const int buf = sd / TC_GROUP, c = c0 + sd;
          if (buf != mine) continue;
          if (c >= n_chunks) break;
          const int g = c / TC_GROUP;
          if (S.bad || !umma::mbar_wait(&S.full_z[sd], (c0 / TC_S) & 1, TC_WAIT) ||
              !umma::mbar_wait(&S.full_a[sd], (c0 / TC_S) & 1, TC_WAIT) ||
              (sd % TC_GROUP == 0 && !umma::mbar_wait(&S.empty_acc[buf], ((g >> 1) & 1) ^ 1, TC_WAIT))) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          const uint32_t d = tmem + TC_COL_ACC + (uint32_t)(buf * TC_NMAX);
          const uint32_t a = tmem + TC_COL_A + (uint32_t)(sd * TC_A_COLS);
          const uint64_t bd = b_desc0 + (uint64_t)sd * b_stage16;
          // small cross terms first, then hi*hi, so the accumulator is still small
          // while the 2^-11-sized terms are added; an accumulator's first group
          // starts from zero, later ones from the residual the drain left
          const uint32_t first = (c0 == 0 && sd % TC_GROUP == 0) ? 0u : 1u;
          const uint32_t pa[3] = {a, a + A_LO, a};
          const uint64_t pb[3] = {bd + b_lo16, bd, bd};
#pragma unroll
          for (int pass = 0; pass < 3; ++pass)
#pragma unroll
            for (int ks = 0; ks < TC_K / 16; ++ks)
              umma::mma_f16_tmem_a(d, pa[pass] + (uint32_t)(32 * (ks / 2) + 8 * (ks % 2)), pb[pass] + (uint64_t)(ks * 2), idesc,
                                   (pass == 0 && ks == 0) ? first : 1u);
          umma::mma_commit(&S.empty[sd]);
          if (sd % TC_GROUP == TC_GROUP - 1 || c == n_chunks - 1) umma::mma_commit(&S.full_acc[buf]);
        }
      }
      if (!ok) S.bad = 1;
      // every MMA this thread issued has finished once mma_done completes
      umma::mma_commit(&S.mma_done);
      if (!umma::mbar_wait(&S.mma_done, 0, TC_WAIT)) S.bad = 1;
    }
  } else if (warp < TC_DRAIN_WARPS) {
    // ---- drain: accumulator of group g -> compensated register sums.  Warp w
    // owns lane quadrant w % 4 and the 16-column blocks TC_DRAIN_PAR i + w / 4
    // (i < 2): s += acc by Fast2Sum on packed FP32 pairs, the rounding residual
    // goes back into the accumulator.  Four warps per quadrant keep a drain
    // short: the next group on this accumulator waits for it
    const int par = warp >> 2;
    constexpr int NB = TC_NMAX / 16 / TC_DRAIN_PAR;  // column blocks per warp
    uint64_t sp[NB][8];  // column pairs of the sums
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int k = 0; k < 8; ++k) sp[i][k] = 0ull;
    bool ok = true;
    for (int g = 0; g < n_groups; ++g) {
      const int buf = g & 1;
      if (!warp_wait(&S.full_acc[buf], (g >> 1) & 1, &S.bad)) {
        ok = false;
        break;
      }
      umma::fence_after_sync();
#pragma unroll
      for (int i = 0; i < NB; ++i) {
        const int cb = 16 * (TC_DRAIN_PAR * i + par);
        if (cb < n) {
          uint32_t v[16];  // accumulator in, residual out
          const uint32_t col = tmem + lanes + TC_COL_ACC + (uint32_t)(buf * TC_NMAX + cb);
          umma::tmem_ld_32x32b_x16(col, v);
          umma::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            // Fast2Sum: t = s + a, e = a - (t - s), exact while |s| >= |a|; when
            // a 64-atom partial outweighs the running sum the residual may lose
            // about an ulp of the partial (~1e-6), far inside the error bounds
            const uint64_t s2 = sp[i][k];
            const uint64_t a2 = pk2(__uint_as_float(v[2 * k]), __uint_as_float(v[2 * k + 1]));
            const uint64_t t2 = add2(s2, a2);
            const uint64_t e2 = sub2(a2, sub2(t2, s2));
            sp[i][k] = t2;
            float e0, e1;
            upk2(e2, e0, e1);
            v[2 * k] = __float_as_uint(e0);
            v[2 * k + 1] = __float_as_uint(e1);
          }
          umma::tmem_st_32x32b_x16(col, v);
        }
      }
      umma::tmem_st_wait();
      umma::fence_before_sync();
      __syncwarp();
      if (lane == 0) umma::mbar_arrive(&S.empty_acc[buf]);
    }
    if (ok && n_groups > 0) {
      // epilogue: the sums into the D staging area, rows of n + 1 floats (the
      // ring is idle: every copy was consumed by an MMA that completed before
      // the last group's commit)
      const int DP = n + 1;
      float* D = reinterpret_cast<float*>(ring);
      const int row = 32 * (warp & 3) + lane;
#pragma unroll
      for (int i = 0; i < NB; ++i) {
        const int cb = 16 * (TC_DRAIN_PAR * i + par);
        if (cb < n)
#pragma unroll
          for (int k = 0; k < 8; ++k) upk2(sp[i][k], D[row * DP + cb + 2 * k], D[row * DP + cb + 2 * k + 1]);
      }
    }
    if (!ok) S.bad = 1;
  } else {
    // ---- builders: A(c) = the chunk's W products into tensor-memory stage c % TC_S.
    // Thread = A lane L = 32 (warp % 4) + lane: complex row r = L / 2 (nx offset
    // r % 8, ny offset r / 8), variant v = L % 2 (0: [Wr, -Wi], 1: [Wi, Wr]);
    // the row's atoms 16 u .. 16 u + 15, u = (warp - TC_BUILD_WARP0) / 4
    const int L = 32 * (warp & 3) + lane;
    const int r = L >> 1, v = L & 1, m = r & 7, yo = r >> 3;
    const int u = (warp - TC_BUILD_WARP0) >> 2;
    for (int c = 0; c < n_chunks; ++c) {
      const int as = c % TC_S;
      // X/Y of chunk c landed; the stage's copies landing implies the MMAs of
      // chunk c - TC_S finished (the producer waited for them), so the A stage
      // in tensor memory is free too
      if (!warp_wait(&S.full_z[as], (c / TC_S) & 1, &S.bad)) {
        S.bad = 1;
        break;
      }
      const unsigned char* st = ring + (size_t)as * zstage + 2 * zhalf;
      const float4* X4 = reinterpret_cast<const float4*>(st);
      const float4* Y4 = reinterpret_cast<const float4*>(st + TC_XB);
      uint32_t hl[32];  // hi of the 16 atoms, then lo
#pragma unroll
      for (int pp = 0; pp < 8; ++pp) {
        const int p = 8 * u + pp;
        const float4 x = X4[p * 16 + m * 2 + v];  // (ar, ai) of atoms 2p, 2p + 1
        const float4 y = Y4[p * 8 + yo];          // (yr, yi) of atoms 2p, 2p + 1
        // (ar + i ai) conj(yr + i yi)
        tc_split2(fmaf(x.x, y.x, x.y * y.y), fmaf(x.y, y.x, -(x.x * y.y)), hl[2 * pp], hl[16 + 2 * pp]);
        tc_split2(fmaf(x.z, y.z, x.w * y.w), fmaf(x.w, y.z, -(x.z * y.w)), hl[2 * pp + 1], hl[17 + 2 * pp]);
      }
      umma::tmem_st_32x32b_x32(tmem + lanes + TC_COL_A + (uint32_t)(as * TC_A_COLS + 32 * u), hl);
      umma::tmem_st_wait();
      umma::fence_before_sync();
      __syncwarp();
      if (lane == 0) umma::mbar_arrive(&S.full_a[as]);
    }
  }

  __syncthreads();
  if (S.bad) {
    // copies still in flight land before the block exits
    // (the last copy issued into each stage; earlier ones were waited for)
    if (tid == 32 * TC_PRODUCER_WARP)
      for (int c = std::max(0, S.z_issued - TC_S); c < S.z_issued; ++c)
        umma::mbar_wait(&S.full_z[c % TC_S], (c / TC_S) & 1, TC_WAIT);
    if (tid == 0) atomicExch(err, 1);
  } else if (n_groups > 0) {
    const int DP = n + 1;
    const float* D = reinterpret_cast<const float*>(ring);
    const int32_t* E = entry_k + T.entry0;
    float2* out = rho + (int64_t)(frame0 + fl) * n_k;
    for (int e = tid; e < TC_ROWS * n; e += TC_THREADS) {
      const int k = E[e];
      if (k >= 0) {
        const int r = e / n, col = e % n;
        out[k] = make_float2(D[(2 * r) * DP + col], D[(2 * r + 1) * DP + col]);
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, TC_TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// host: tile plan over the shell-sorted vector list, launches per frame batch
// ---------------------------------------------------------------------------

static bool tc_half_space(int nx, int ny, int nz) {
  return nz > 0 || (nz == 0 && (ny > 0 || (ny == 0 && nx > 0)));
}

TcPlan* tc_plan_build(const std::vector<int32_t>& kvec) {
  const int nk = (int)(kvec.size() / 3);
  int nmax = 0;
  for (int v : kvec) nmax = std::max(nmax, std::abs(v));
  const int W = 2 * nmax + 1, H = nmax + 1;
  std::vector<int32_t> index((size_t)W * W * H, -1);
  for (int k = 0; k < nk; ++k) {
    const int x = kvec[3 * k] + nmax, y = kvec[3 * k + 1] + nmax, z = kvec[3 * k + 2];
    AMDAT_REQUIRE(z >= 0 && tc_half_space(kvec[3 * k], kvec[3 * k + 1], z), "lattice vector outside the half space");
    index[((size_t)x * W + y) * H + z] = k;
  }
  // nz windows: one window of the smallest multiple of 16 covering 0..nmax, or
  // windows of TC_NMAX; each tile's width is trimmed to its rows' extent
  const int nzw = std::min(TC_NMAX, (nmax + 1 + 15) / 16 * 16);
  const int n_zblk = (nmax + nzw) / nzw;
  std::vector<TcTile> tiles;
  std::vector<int32_t> entries;
  int64_t computed = 0;
  for (int x0 = -nmax; x0 <= nmax; x0 += 8)
    for (int y0 = -nmax; y0 <= nmax; y0 += 8)
      for (int zb = 0; zb < n_zblk; ++zb) {
        int last = -1;
        for (int r = 0; r < TC_ROWS; ++r)
          for (int c = 0; c < nzw; ++c) {
            const int nx = x0 + (r & 7), ny = y0 + (r >> 3), nz = zb * nzw + c;
            if (nx > nmax || ny > nmax || nz > nmax) continue;
            if (index[((size_t)(nx + nmax) * W + (ny + nmax)) * H + nz] >= 0) last = std::max(last, c);
          }
        if (last < 0) continue;
        const int n = (last + 1 + 15) / 16 * 16;
        const int32_t e0 = (int32_t)entries.size();
        for (int r = 0; r < TC_ROWS; ++r)
          for (int c = 0; c < n; ++c) {
            const int nx = x0 + (r & 7), ny = y0 + (r >> 3), nz = zb * nzw + c;
            int k = -1;
            if (nx <= nmax && ny <= nmax && nz <= nmax)
              k = index[((size_t)(nx + nmax) * W + (ny + nmax)) * H + nz];
            entries.push_back(k);
          }
        tiles.push_back(TcTile{x0, y0, zb, e0, n, 0, 0, 0});
        computed += (int64_t)TC_ROWS * n;
      }
  AMDAT_REQUIRE(entries.size() < (size_t)INT32_MAX, "lattice too large for the tensor-core tiling");
  auto* p = new TcPlan();
  p->n_tiles = (int32_t)tiles.size();
  p->n_zblk = n_zblk;
  p->nzw = nzw;
  p->nmax = nmax;
  p->entries = computed;
  p->host_tiles = tiles;
  p->tiles.reserve(std::max<size_t>(tiles.size(), 1));
  p->entry_k.reserve(std::max<size_t>(entries.size(), 1));
  if (!tiles.empty()) {
    AMDAT_CUDA(cudaMemcpy(p->tiles.ptr, tiles.data(), tiles.size() * sizeof(TcTile), cudaMemcpyHostToDevice));
    AMDAT_CUDA(cudaMemcpy(p->entry_k.ptr, entries.data(), entries.size() * 4, cudaMemcpyHostToDevice));
  }
  return p;
}

void tc_plan_free(TcPlan* p) { delete p; }

int64_t tc_plan_entries(const TcPlan& p) { return p.entries; }

// rho[f][k] for frames 0..n_frames-1 of fx ([n_frames][n_list] fixed-point phases)
void rhok_tc_run(amdat_ctx* ctx, const TcPlan& P, const int4* fx, int32_t n_list, int32_t n_frames,
                 int32_t n_k, float2* rho) {
  if (P.n_tiles == 0 || n_list == 0 || n_frames == 0) return;
  const int32_t n_chunks = (int32_t)ceil_div(n_list, TC_J);
  const int32_t n_blk = 2 * P.nmax / 8 + 1;  // 8-index blocks from -nmax covering the tiles
  const size_t zblob = (size_t)2 * P.nzw * TC_K * 2;
  const size_t z_frame = (size_t)P.n_zblk * n_chunks * zblob;
  const size_t xy_frame = (size_t)n_blk * n_chunks * TC_XYB;
  const size_t per_frame = z_frame + xy_frame;
  // frame batches bound the operand buffers to ~1 GB
  const int32_t batch = (int32_t)std::max<size_t>(1, std::min<size_t>(n_frames, (size_t)(1u << 30) / per_frame));
  unsigned char* zbuf = ctx->scratch.reserve(per_frame * batch + 256);
  float2* xybuf = reinterpret_cast<float2*>(zbuf + z_frame * batch);
  int* d_err = (int*)(zbuf + per_frame * batch);
  AMDAT_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  // the ring beside the barrier header (1024 bytes of alignment slack); the
  // epilogue stages D (128 rows of n + 1 floats) in the idle ring
  const uint32_t zstage = tc_zstage(P.nzw);
  const size_t shm = 1024 + TC_HDR + (size_t)TC_S * zstage;
  AMDAT_REQUIRE(shm <= TC_SMEM_MAX, "nz window too wide for the tensor-core ring");
  AMDAT_REQUIRE((size_t)TC_S * zstage >= sizeof(float) * TC_M * (P.nzw + 1), "ring too small for the D staging");
  AMDAT_CUDA(cudaFuncSetAttribute(rhok_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  for (int32_t f0 = 0; f0 < n_frames; f0 += batch) {
    const int32_t nb = std::min(batch, n_frames - f0);
    zgen_kernel<<<(unsigned)(nb * P.n_zblk * n_chunks), 256, 0, ctx->stream>>>(
        fx + (int64_t)f0 * n_list, n_list, n_chunks, P.n_zblk, P.nzw, zbuf);
    check_launch("zgen_kernel");
    count_launch(ctx);
    xygen_kernel<<<(unsigned)(nb * n_blk * n_chunks), 256, 0, ctx->stream>>>(
        fx + (int64_t)f0 * n_list, n_list, n_chunks, n_blk, P.nmax, xybuf);
    check_launch("xygen_kernel");
    count_launch(ctx);
    KernelTimer kt(ctx, "rhok_tc_kernel");
    dim3 grid((unsigned)P.n_tiles, (unsigned)nb);
    rhok_tc_kernel<<<grid, TC_THREADS, shm, ctx->stream>>>(n_list, n_chunks, P.n_zblk, P.nzw, n_blk, P.nmax,
                                                          P.tiles.ptr, P.entry_k.ptr, zbuf, xybuf, f0, n_k,
                                                          rho, d_err);
    check_launch("rhok_tc_kernel");
    count_launch(ctx);
  }
  int h_err = 0;
  AMDAT_CUDA(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h_err) throw Error(AMDAT_ERR_TIMEOUT, "tensor-core rho_k: a bounded wait timed out");
}

}  // namespace amdat
