// Tensor-core (tcgen05) Fourier densities over the whole half-space lattice.
//
// rho[(nx,ny), nz] = sum_j W_j(nx,ny) Z_j(nz), W = X(nx) Y(ny), is a complex
// GEMM with the atoms as the reduction axis.  As a real GEMM per tile:
//   A (128 x 2J): rows 0..63   = [Wr, -Wi] of 64 (nx,ny) rows (8 nx x 8 ny),
//                 rows 64..127 = [Wi,  Wr]           (k = 2j, 2j+1 per atom j)
//   B (  n x 2J): [Zr, Zi] for n consecutive nz (n <= 128, a multiple of 16,
//                 sized per tile to the nz extent of its 64 rows)
//   D = A B^T  (128 x n): rows 0..63 = Re rho, rows 64..127 = Im rho.
// Operands are FP16 split into hi + lo parts (x = hi + lo to ~2^-22), and each
// chunk of 32 atoms runs three tcgen05.mma passes, hi*lo + lo*hi + hi*hi (small
// terms first), accumulating in FP32 tensor memory.  The tensor core's FP32
// accumulation drops low bits as the accumulator grows, so an accumulation
// never spans more than TC_GROUP chunks (64 atoms): the accumulator is then
// drained into Kahan-compensated sums that also live in tensor memory.  The
// phases are the exact fixed-point phases of the FP32 kernels (fraction of the
// box in units of 2^-31 turns).
//
// Per frame batch, zgen_kernel precomputes the B operands (Z hi/lo in the
// K-major 128-byte-swizzled layout, one blob per (frame, nz window, chunk)).  The
// main kernel is warp-specialised, one CTA per SM, 512 TMEM columns:
//   warps 0-3   drain: TMEM accumulator -> Kahan (s, c) columns, then the epilogue
//   warp 4      producer: bulk copies (cp.async.bulk) of Z hi/lo and the X/Y
//               phase tables of each chunk into a 3-stage ring
//   warps 5-6   MMA issuers, one per accumulator (alternate 64-atom groups):
//               12 tcgen05.mma per chunk
//   warps 7-22  builders: the A operand of the chunk (W = X Y products, FP16
//               split, swizzled K-major stores) into the same ring stage
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
#include "tc_tiles.h"
#include "umma.cuh"

namespace amdat {

constexpr int TC_J = 32;                      // atoms per chunk
constexpr int TC_K = 2 * TC_J;                // real K per chunk
constexpr int TC_ROWS = 64;                   // complex rows (8 nx x 8 ny)
constexpr int TC_NMAX = 128;                  // widest nz window (MMA N)
constexpr int TC_M = 2 * TC_ROWS;             // MMA M = 128
constexpr int TC_GROUP = 2;                   // chunks per tensor-memory accumulation
constexpr int TC_S = 3;                       // ring stages (Z, X, Y and the A operand of one chunk)
constexpr int TC_PRODUCER_WARP = 4;
constexpr int TC_MMA_WARP = 5;                // warps 5 and 6: one per accumulator
constexpr int TC_MMA_WARPS = 2;
constexpr int TC_BUILD_WARP0 = TC_MMA_WARP + TC_MMA_WARPS;
constexpr int TC_BUILDERS = 512;              // 16 builder warps
constexpr int TC_BUILD_GROUP = TC_BUILDERS / 2;  // two groups of 8 warps, alternate chunks
constexpr int TC_DRAINERS = 128;              // warps 0-3, one per TMEM lane quadrant
constexpr int TC_THREADS = 32 * TC_BUILD_WARP0 + TC_BUILDERS;  // 736
constexpr uint32_t TC_A_BYTES = TC_M * TC_K * 2;      // 16 KB (one of hi / lo)
constexpr uint32_t TC_ZHALF = TC_NMAX * TC_K * 2;     // 16 KB (one of hi / lo, widest window)
constexpr uint32_t TC_XYB = TC_J * 8 * sizeof(float2);  // 2 KB: 8 phases of 32 atoms (X or Y)
constexpr uint32_t TC_STAGE = 2 * TC_ZHALF + 2 * TC_XYB;  // Z hi, Z lo, X, Y
constexpr uint32_t TC_WAIT = 1u << 19;                // try_wait calls of <= 1 us (~0.5 s bound)
// tensor-memory columns: two accumulators, then the Kahan sums and compensations
constexpr uint32_t TC_COL_ACC = 0, TC_COL_S = 2 * TC_NMAX, TC_COL_C = 3 * TC_NMAX;
constexpr uint32_t TC_TMEM_COLS = 4 * TC_NMAX;        // 512


struct TcSmem {
  unsigned char z[TC_S][TC_STAGE];      // [stage] Z hi, Z lo, X, Y; the epilogue stages D here
  unsigned char a[TC_S][2][TC_A_BYTES];  // [stage][hi|lo]
  uint64_t full_z[TC_S], full_a[TC_S];  // bulk copies landed / A built
  uint64_t empty[TC_S];                 // the stage's MMAs finished (one commit per chunk)
  uint64_t full_acc[2], empty_acc[2];
  uint64_t mma_done;
  uint32_t tmem;
  volatile int bad;        // any role gave up
  int build_stop[2][2];    // [group][chunk parity]: written by the group's first thread before its barrier
  int z_issued, z_landed;  // bulk copies issued / seen complete
};
static_assert(sizeof(float) * TC_M * (TC_NMAX + 1) <= sizeof(((TcSmem*)0)->z), "D staging must fit the Z ring");
// operands use the 128-byte-swizzled K-major layout: 128-byte rows, 1024-byte aligned tiles
static_assert(TC_K * 2 == 128, "one chunk's K must fill a 128-byte swizzle row");
static_assert(TC_STAGE % 1024 == 0 && TC_ZHALF % 1024 == 0 && TC_A_BYTES % 1024 == 0,
              "every operand tile must start on a 1024-byte boundary");

__device__ __forceinline__ void tc_split(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(__fsub_rn(x, __half2float(hi)));
}

__device__ __forceinline__ void tc_phase(int32_t ph, float* s, float* c) {
  sincospif(__fmul_rn((float)ph, 9.313225746154785e-10f), s, c);  // ph * 2^-30 * pi
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

// X/Y table of a 32-atom block: 8 rows (lattice index offset m) of 16 chunks
// of 16 bytes, chunk = two atoms' (cos, sin).  Atom pair p = j / 2 of row m
// sits in chunk 16 m + ((m + p) & 15): a builder warp's 128-bit loads (8
// rows x 4 atom quads, or one row broadcast) are then free of bank conflicts.
// Returns the float2 index of (atom j, row m).
__device__ __forceinline__ int xy_slot(int j, int m) { return 2 * (16 * m + ((m + (j >> 1)) & 15)) + (j & 1); }

// X and Y phase tables of one frame batch: for axis a (0 = x, 1 = y), block b
// of 8 lattice indices (n = -nmax + 8 b + m) and chunk c of 32 atoms, a 2 KB
// block at ((f * 2 + a) * n_blk + b) * n_chunks + c holding exp(i 2 pi n q_a)
__global__ void __launch_bounds__(256)
    xygen_kernel(const int4* __restrict__ fx, int32_t n_list, int32_t n_chunks, int32_t n_blk,
                 int32_t nmax, float2* __restrict__ xybuf) {
  const int blk = blockIdx.x;  // ((f * 2 + axis) * n_blk + b) * n_chunks + c
  const int c = blk % n_chunks;
  const int b = (blk / n_chunks) % n_blk;
  const int axis = (blk / (n_chunks * n_blk)) & 1;
  const int f = blk / (n_chunks * n_blk * 2);
  float2* out = xybuf + (size_t)blk * (TC_J * 8);
  const int4* F = fx + (int64_t)f * n_list;
  for (int e = threadIdx.x; e < TC_J * 8; e += blockDim.x) {
    const int j = e >> 3, m = e & 7;
    const int a = c * TC_J + j;
    float sn = 0.f, cs = 0.f;
    if (a < n_list) {
      const int32_t q = axis ? F[a].y : F[a].x;
      const int32_t n = -nmax + 8 * b + m;
      tc_phase((int32_t)((uint32_t)n * (uint32_t)q), &sn, &cs);
    }
    out[xy_slot(j, m)] = make_float2(cs, sn);
  }
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
                   int32_t nmax, const TcTile* __restrict__ tiles, const int32_t* __restrict__ entry_k,
                   const unsigned char* __restrict__ zbuf, const float2* __restrict__ xybuf,
                   int32_t frame0, int32_t n_k, float2* __restrict__ rho, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const TcTile T = tiles[blockIdx.x];
  const int fl = blockIdx.y;  // frame within the batch
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = T.n;
  const uint32_t zhalf = (uint32_t)nzw * TC_K * 2;
  const unsigned char* Z = zbuf + ((size_t)fl * n_zblk + T.zblk) * (size_t)n_chunks * 2 * zhalf;
  const float2* XT = xybuf + (((size_t)fl * 2 + 0) * n_blk + (T.nx0 + nmax) / 8) * (size_t)n_chunks * (TC_J * 8);
  const float2* YT = xybuf + (((size_t)fl * 2 + 1) * n_blk + (T.ny0 + nmax) / 8) * (size_t)n_chunks * (TC_J * 8);
  const int n_groups = (n_chunks + TC_GROUP - 1) / TC_GROUP;

  if (tid == 0) {
    for (int s = 0; s < TC_S; ++s) {
      umma::mbar_init(&S.full_z[s], 1);
      umma::mbar_init(&S.full_a[s], TC_BUILD_GROUP);  // one group builds each chunk
      umma::mbar_init(&S.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(&S.full_acc[b], 1);
      umma::mbar_init(&S.empty_acc[b], TC_DRAINERS);
    }
    umma::mbar_init(&S.mma_done, TC_MMA_WARPS);
    umma::fence_mbarrier_init();
    S.bad = 0;
    S.build_stop[0][0] = S.build_stop[0][1] = S.build_stop[1][0] = S.build_stop[1][1] = 0;
    S.z_issued = 0;
    S.z_landed = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(&S.tmem, TC_TMEM_COLS);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = S.tmem;

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
        const unsigned char* src = Z + (size_t)c * 2 * zhalf;
        umma::mbar_expect_tx(&S.full_z[s], 2u * n * TC_K * 2 + 2 * TC_XYB);
        umma::bulk_g2s(S.z[s], src, (uint32_t)n * TC_K * 2, &S.full_z[s]);
        umma::bulk_g2s(S.z[s] + TC_ZHALF, src + zhalf, (uint32_t)n * TC_K * 2, &S.full_z[s]);
        umma::bulk_g2s(S.z[s] + 2 * TC_ZHALF, XT + (size_t)c * (TC_J * 8), TC_XYB, &S.full_z[s]);
        umma::bulk_g2s(S.z[s] + 2 * TC_ZHALF + TC_XYB, YT + (size_t)c * (TC_J * 8), TC_XYB, &S.full_z[s]);
      }
      S.z_issued = c;
    }
  } else if (warp >= TC_MMA_WARP && warp < TC_MMA_WARP + TC_MMA_WARPS) {
    // ---- MMA issuers: warp TC_MMA_WARP + b issues the groups of accumulator b
    // (even / odd groups), so two threads keep the tensor pipe fed; the two
    // accumulators are independent, and each chunk's stage is read by one issuer
    const int mine = warp - TC_MMA_WARP;
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_f16_f32(TC_M, n);
      // descriptors are built once: a descriptor's address field is the byte
      // address >> 4 (14 bits, all of shared memory), so moving to another
      // stage, the lo half (both 1024-byte aligned) or the next k-step (32 B
      // inside the swizzled 128-byte rows) adds a constant
      const uint64_t a_desc0 = umma::smem_desc_sw128(umma::smem_addr(S.a[0][0]));
      const uint64_t b_desc0 = umma::smem_desc_sw128(umma::smem_addr(S.z[0]));
      constexpr uint32_t A_STAGE16 = (2 * TC_A_BYTES) >> 4, A_LO16 = TC_A_BYTES >> 4;
      constexpr uint32_t B_STAGE16 = TC_STAGE >> 4, B_LO16 = TC_ZHALF >> 4;
      bool ok = true;
      for (int c = 0; c < n_chunks; ++c) {
        const int sz = c % TC_S, sa = sz, g = c / TC_GROUP, buf = g & 1;
        if (buf != mine) continue;
        if (S.bad || !umma::mbar_wait(&S.full_z[sz], (c / TC_S) & 1, TC_WAIT)) {
          ok = false;
          break;
        }
        atomicMax(&S.z_landed, c + 1);
        if (!umma::mbar_wait(&S.full_a[sa], (c / TC_S) & 1, TC_WAIT) ||
            (c % TC_GROUP == 0 && !umma::mbar_wait(&S.empty_acc[buf], ((g >> 1) & 1) ^ 1, TC_WAIT))) {
          ok = false;
          break;
        }
        umma::fence_after_sync();
        const uint32_t d = tmem + TC_COL_ACC + (uint32_t)(buf * TC_NMAX);
        const uint64_t ad = a_desc0 + (uint64_t)(sa * A_STAGE16), bd = b_desc0 + (uint64_t)(sz * B_STAGE16);
        // small cross terms first, then hi*hi, so the accumulator is still small
        // while the 2^-11-sized terms are added
        const uint64_t pa[3] = {ad, ad + A_LO16, ad}, pb[3] = {bd + B_LO16, bd, bd};
#pragma unroll
        for (int pass = 0; pass < 3; ++pass)
#pragma unroll
          for (int ks = 0; ks < TC_K / 16; ++ks)
            umma::mma_f16(d, pa[pass] + (uint64_t)(ks * 2), pb[pass] + (uint64_t)(ks * 2), idesc,
                          (c % TC_GROUP == 0 && pass == 0 && ks == 0) ? 0u : 1u);
        umma::mma_commit(&S.empty[sz]);
        if (c % TC_GROUP == TC_GROUP - 1 || c == n_chunks - 1) umma::mma_commit(&S.full_acc[buf]);
      }
      if (!ok) S.bad = 1;
      // every MMA this thread issued has finished once mma_done completes
      umma::mma_commit(&S.mma_done);
      if (!umma::mbar_wait(&S.mma_done, 0, TC_WAIT)) S.bad = 1;
    }
  } else if (warp < 4) {
    // ---- drain: accumulator of group g -> Kahan sums (s, c) in tensor memory
    const uint32_t lanes = (uint32_t)(32 * warp) << 16;
    bool ok = true;
    for (int g = 0; g < n_groups; ++g) {
      const int buf = g & 1;
      if (!warp_wait(&S.full_acc[buf], (g >> 1) & 1, &S.bad)) {
        ok = false;
        break;
      }
      umma::fence_after_sync();
      for (int cb = 0; cb < n; cb += 16) {
        uint32_t v[16], s[16], cc[16];
        umma::tmem_ld_32x32b_x16(tmem + lanes + TC_COL_ACC + (uint32_t)(buf * TC_NMAX + cb), v);
        if (g > 0) {
          umma::tmem_ld_32x32b_x16(tmem + lanes + TC_COL_S + (uint32_t)cb, s);
          umma::tmem_ld_32x32b_x16(tmem + lanes + TC_COL_C + (uint32_t)cb, cc);
        }
        umma::tmem_ld_wait();
        if (g == 0) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            s[i] = v[i];
            cc[i] = 0u;
          }
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float sv = __uint_as_float(s[i]), cv = __uint_as_float(cc[i]);
            const float y = __fsub_rn(__uint_as_float(v[i]), cv);
            const float t = __fadd_rn(sv, y);
            cc[i] = __float_as_uint(__fsub_rn(__fsub_rn(t, sv), y));
            s[i] = __float_as_uint(t);
          }
        }
        umma::tmem_st_32x32b_x16(tmem + lanes + TC_COL_S + (uint32_t)cb, s);
        umma::tmem_st_32x32b_x16(tmem + lanes + TC_COL_C + (uint32_t)cb, cc);
      }
      umma::tmem_st_wait();
      umma::fence_before_sync();
      umma::mbar_arrive(&S.empty_acc[buf]);
    }
    if (ok && n_groups > 0) {
      // epilogue: s - c into the D staging area (the Z ring is idle: every copy
      // was consumed by an MMA that completed before the last group's commit)
      constexpr int DP = TC_NMAX + 1;
      float* D = reinterpret_cast<float*>(S.z[0]);
      const int row = 32 * warp + lane;
      for (int cb = 0; cb < n; cb += 16) {
        uint32_t s[16], cc[16];
        umma::tmem_ld_32x32b_x16(tmem + lanes + TC_COL_S + (uint32_t)cb, s);
        umma::tmem_ld_32x32b_x16(tmem + lanes + TC_COL_C + (uint32_t)cb, cc);
        umma::tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 16; ++i)
          D[row * DP + cb + i] = __fsub_rn(__uint_as_float(s[i]), __uint_as_float(cc[i]));
      }
    }
    if (!ok) S.bad = 1;
  } else {
    // ---- builders: A(c) = W products of the streamed X/Y tables into stage c % TC_S.
    // Two groups of 8 warps build alternate chunks (group g: chunks c with c % 2 == g),
    // so the wait / build / fence chain of one chunk overlaps the next one's.
    const int btid = tid - 32 * TC_BUILD_WARP0;
    const int grp = btid / TC_BUILD_GROUP, gtid = btid % TC_BUILD_GROUP, gw = gtid >> 5;
    for (int c = grp; c < n_chunks; c += 2) {
      const int sa = c % TC_S, sz = sa, par = (c >> 1) & 1;
      // the group's first thread decides for the group (X/Y of chunk c landed;
      // the stage's copies landing implies its previous MMAs finished, since the
      // producer waited for them, so the A half of the stage is free too); the
      // flag alternates with the group's chunk parity so a slow reader of one
      // chunk never sees the next one's decision
      if (gtid == 0) {
        const bool go = !S.bad && umma::mbar_wait(&S.full_z[sz], (c / TC_S) & 1, TC_WAIT);
        S.build_stop[grp][par] = go ? 0 : 1;
      }
      __syncwarp();
      if (grp == 0)
        umma::named_barrier(1, TC_BUILD_GROUP);
      else
        umma::named_barrier(2, TC_BUILD_GROUP);
      if (*(volatile int*)&S.build_stop[grp][par]) {
        if (gtid == 0) S.bad = 1;
        break;
      }
      // A operand: thread = complex row r (nx = lane % 8, ny = warp of the group)
      // and the atom octet o (atom quads 2o, 2o+1): four 128-bit loads each of X
      // and Y, eight 128-bit stores (hi and lo of the real row [Wr, -Wi] and of
      // the imaginary row [Wi, Wr] for both quads), all free of bank conflicts
      const float4* X4 = reinterpret_cast<const float4*>(S.z[sz] + 2 * TC_ZHALF);
      const float4* Y4 = X4 + TC_J * 8 / 2;
      const int m = lane & 7, rg = gw, o = lane >> 3;
      const int r = rg * 8 + m;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = 2 * o + h;
        const float4 xa = X4[16 * m + ((m + 2 * q) & 15)], xb = X4[16 * m + ((m + 2 * q + 1) & 15)];
        const float4 ya = Y4[16 * rg + ((rg + 2 * q) & 15)], yb = Y4[16 * rg + ((rg + 2 * q + 1) & 15)];
        const float xr[4] = {xa.x, xa.z, xb.x, xb.z}, xi[4] = {xa.y, xa.w, xb.y, xb.w};
        const float yr[4] = {ya.x, ya.z, yb.x, yb.z}, yi[4] = {ya.y, ya.w, yb.y, yb.w};
        uint32_t hre[4], lre[4], him[4], lim[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float wr = fmaf(xr[a], yr[a], -xi[a] * yi[a]);
          const float nwi = fmaf(-xr[a], yi[a], -xi[a] * yr[a]);  // -Im W
          // hi = fp16(w), lo = fp16(w - hi) of the real row (Wr, -Wi); the
          // imaginary row (Wi, Wr) is the same pair swapped with the first
          // element negated (round to nearest is symmetric)
          const __half2 hi = __floats2half2_rn(wr, nwi);
          const float2 hb = __half22float2(hi);
          const __half2 lo = __floats2half2_rn(__fsub_rn(wr, hb.x), __fsub_rn(nwi, hb.y));
          hre[a] = *reinterpret_cast<const uint32_t*>(&hi);
          lre[a] = *reinterpret_cast<const uint32_t*>(&lo);
          him[a] = __byte_perm(hre[a], 0, 0x1032) ^ 0x00008000u;
          lim[a] = __byte_perm(lre[a], 0, 0x1032) ^ 0x00008000u;
        }
        const uint32_t o_re = (uint32_t)(r * 128 + ((q ^ (r & 7)) << 4));  // K = 8q..8q+7, 128-byte swizzle
        const uint32_t o_im = o_re + (uint32_t)TC_ROWS * 128;                  // row r + 64, same swizzle
        *reinterpret_cast<uint4*>(S.a[sa][0] + o_re) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
        *reinterpret_cast<uint4*>(S.a[sa][1] + o_re) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
        *reinterpret_cast<uint4*>(S.a[sa][0] + o_im) = make_uint4(him[0], him[1], him[2], him[3]);
        *reinterpret_cast<uint4*>(S.a[sa][1] + o_im) = make_uint4(lim[0], lim[1], lim[2], lim[3]);
      }
      umma::fence_proxy_async_smem();
      umma::mbar_arrive(&S.full_a[sa]);
    }
  }

  __syncthreads();
  if (S.bad) {
    // copies still in flight land before the block exits
    if (tid == 32 * TC_PRODUCER_WARP)
      for (int c = S.z_landed; c < S.z_issued; ++c)
        umma::mbar_wait(&S.full_z[c % TC_S], (c / TC_S) & 1, TC_WAIT);
    if (tid == 0) atomicExch(err, 1);
  } else if (n_groups > 0) {
    constexpr int DP = TC_NMAX + 1;
    const float* D = reinterpret_cast<const float*>(S.z[0]);
    const int32_t* E = entry_k + T.entry0;
    float2* out = rho + (int64_t)(frame0 + fl) * n_k;
    for (int e = tid; e < TC_ROWS * n; e += TC_THREADS) {
      const int k = E[e];
      if (k >= 0) {
        const int r = e / n, col = e % n;
        out[k] = make_float2(D[r * DP + col], D[(TC_ROWS + r) * DP + col]);
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
  const size_t xy_frame = (size_t)2 * n_blk * n_chunks * TC_XYB;
  const size_t per_frame = z_frame + xy_frame;
  // frame batches bound the operand buffers to ~1 GB
  const int32_t batch = (int32_t)std::max<size_t>(1, std::min<size_t>(n_frames, (size_t)(1u << 30) / per_frame));
  unsigned char* zbuf = ctx->scratch.reserve(per_frame * batch + 256);
  float2* xybuf = reinterpret_cast<float2*>(zbuf + z_frame * batch);
  int* d_err = (int*)(zbuf + per_frame * batch);
  AMDAT_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  const size_t shm = sizeof(TcSmem) + 1024;
  AMDAT_CUDA(cudaFuncSetAttribute(rhok_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  for (int32_t f0 = 0; f0 < n_frames; f0 += batch) {
    const int32_t nb = std::min(batch, n_frames - f0);
    zgen_kernel<<<(unsigned)(nb * P.n_zblk * n_chunks), 256, 0, ctx->stream>>>(
        fx + (int64_t)f0 * n_list, n_list, n_chunks, P.n_zblk, P.nzw, zbuf);
    check_launch("zgen_kernel");
    count_launch(ctx);
    xygen_kernel<<<(unsigned)(nb * 2 * n_blk * n_chunks), 256, 0, ctx->stream>>>(
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
