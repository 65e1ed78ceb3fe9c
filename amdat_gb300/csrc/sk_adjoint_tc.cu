// S(k) adjoint on the tensor cores for lattice densities (no reference
// counterpart; the forward is Structure_Factor, src/structure_factor.cpp:201-320).
//
// For atom j and a tile of 64 (nx, ny) rows x n nz columns (the forward's
// tiling), with c = u_k conj(rho_k) (u_k = 2 w_s / H_s) on the tile's vectors:
//   T_j(row)  = sum_nz c(row, nz)      Z_j(nz)        Z_j(nz) = exp(i 2 pi nz q_z)
//   T'_j(row) = sum_nz nz c(row, nz)   Z_j(nz)
//   dLoss/dr_j = -(2 pi / L) Im sum_row W_j(row) (nx T, ny T, T')   W = X(nx) Y(ny)
// T and T' are GEMMs with the atoms as M: D[atom][2m + {0,1}] = {Re, Im} T_m.
// The kernel is atom-stationary: a CTA keeps Z of its 128 atoms (FP16 hi/lo,
// K = 2 x nz window, re/im interleaved) in shared memory, streams the
// coefficient tiles (C and nz C, FP16 hi/lo, scaled into FP16 range) in
// chunks of 16 nz by bulk copy through a 3-stage ring, runs 12 tcgen05.mma per
// chunk (3 split passes x 2 k-steps x {T, T'}; warp 5 issues the T and warp 6
// the T' MMAs) into one of two TMEM accumulator pairs, and four epilogue warps (one atom per thread) read T and
// T', form W from exact fixed-point phases and add the tile's contribution to
// the atom's Kahan-compensated sums.  Every atom's gradient is written by one
// thread after a fixed sequence of tiles: deterministic.
//
// Warps 0-3: epilogue; warp 4: producer; warps 5-6: MMA issuers (T, T').  Waits are
// bounded; a timeout makes every role stop, wait for its copies and MMAs,
// free tensor memory and set an error word.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.h"
#include "tc_tiles.h"
#include "umma.cuh"

namespace amdat {

constexpr int SA_M = 128;                         // atoms per CTA
constexpr int SA_KC = 32;                         // real K per chunk (16 nz, re/im)
constexpr int SA_N = 128;                         // 64 complex rows -> Re, Im rows
constexpr int SA_STAGES = 3;
constexpr uint32_t SA_BPART = SA_N * SA_KC * 2;   // 8 KB: one of C hi, C lo, C' hi, C' lo
constexpr uint32_t SA_BSTAGE = 4 * SA_BPART;      // 32 KB per chunk
constexpr int SA_ISSUERS = 2;                    // warp 5 issues T, warp 6 issues T'
constexpr int SA_THREADS = 32 * (5 + SA_ISSUERS);  // 224
constexpr uint32_t SA_WAIT = 1u << 19;             // try_wait calls of <= 1 us
constexpr uint32_t SA_TMEM_COLS = 512;             // two (T, T') accumulator pairs

struct SaBars {
  uint64_t full_b[SA_STAGES], empty_b[SA_STAGES];
  uint64_t full_acc[2], empty_acc[2];
  uint64_t mma_done;
  uint32_t tmem;
  volatile int bad;
  int issued, landed;
};

__device__ __forceinline__ void sa_split(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(__fsub_rn(x, __half2float(hi)));
}

__device__ __forceinline__ void sa_phase(int32_t ph, float* s, float* c) {
  sincospif(__fmul_rn((float)ph, 9.313225746154785e-10f), s, c);  // ph * 2^-31 turns
}

// B blobs: for frame f and chunk g (tile t = chunk_tile[g], chunk q), the
// four 128 x 32 K-major parts [C hi | C lo | C' hi | C' lo]:
//   row 2m   (Re T_m): k = 2z -> cr,  k = 2z+1 -> -ci
//   row 2m+1 (Im T_m): k = 2z -> ci,  k = 2z+1 ->  cr
// with (cr, ci) = scale * u_k conj(rho_k) of vector (nx0 + m%8, ny0 + m/8, nz),
// and C' the same times nz (its own scale).
__global__ void __launch_bounds__(256)
    sa_blob_kernel(const float2* __restrict__ rho, int32_t n_k, const float* __restrict__ u,
                   const TcTile* __restrict__ tiles, const int32_t* __restrict__ entry_k,
                   const int32_t* __restrict__ chunk_tile, const int32_t* __restrict__ chunk_q,
                   int32_t n_chunks, int32_t nzw, float scale_c, float scale_cz,
                   unsigned char* __restrict__ blobs) {
  const int g = blockIdx.x, f = blockIdx.y;
  const TcTile T = tiles[chunk_tile[g]];
  const int q = chunk_q[g];
  const float2* R = rho + (int64_t)f * n_k;
  unsigned char* out = blobs + ((size_t)f * n_chunks + g) * SA_BSTAGE;
  // one (row, z) pair per item: both k = 2z, 2z+1 as a half2, for C and C'
  for (int e = threadIdx.x; e < SA_N * (SA_KC / 2); e += blockDim.x) {
    const int r = e / (SA_KC / 2), z = e % (SA_KC / 2);
    const int m = r >> 1, im = r & 1;
    const int zl = q * (SA_KC / 2) + z;  // nz within the tile
    float cr = 0.f, ci = 0.f;
    if (zl < T.n) {
      const int k = entry_k[T.entry0 + m * T.n + zl];
      if (k >= 0) {
        const float2 rk = R[k];
        cr = u[k] * rk.x;
        ci = -u[k] * rk.y;
      }
    }
    const float v0 = im ? ci : cr, v1 = im ? cr : -ci;
    const float nz = (float)(T.zblk * nzw + zl);
    __half h0, l0, h1, l1;
    const uint32_t off = umma::kmajor_offset(r, 2 * z, SA_KC);
    sa_split(v0 * scale_c, h0, l0);
    sa_split(v1 * scale_c, h1, l1);
    *reinterpret_cast<__half2*>(out + off) = __halves2half2(h0, h1);
    *reinterpret_cast<__half2*>(out + SA_BPART + off) = __halves2half2(l0, l1);
    sa_split(v0 * nz * scale_cz, h0, l0);
    sa_split(v1 * nz * scale_cz, h1, l1);
    *reinterpret_cast<__half2*>(out + 2 * SA_BPART + off) = __halves2half2(h0, h1);
    *reinterpret_cast<__half2*>(out + 3 * SA_BPART + off) = __halves2half2(l0, l1);
  }
}

__global__ void __launch_bounds__(SA_THREADS, 1)
    sk_adjoint_tc_kernel(const int4* __restrict__ fx /*[F][n]*/, int32_t n, int32_t zb, int32_t nzw,
                         const TcTile* __restrict__ tiles, const int32_t* __restrict__ tile_list,
                         int32_t n_list_tiles, const int32_t* __restrict__ tile_chunk0,
                         const unsigned char* __restrict__ blobs, int32_t n_chunks, float inv_c,
                         float inv_cz, float scale, int32_t accumulate, float* __restrict__ grad,
                         int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int KA = 2 * nzw;                          // A's K: nz window, re/im interleaved
  const uint32_t a_half = (uint32_t)SA_M * KA * 2;
  unsigned char* A_hi = base;
  unsigned char* A_lo = base + a_half;
  unsigned char* B = base + ((2 * a_half + 1023) & ~1023u);
  SaBars& S = *reinterpret_cast<SaBars*>(B + SA_STAGES * SA_BSTAGE);
  const int f = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int4* F = fx + (int64_t)f * n;
  const unsigned char* Bf = blobs + (size_t)f * n_chunks * SA_BSTAGE;

  if (tid == 0) {
    for (int s = 0; s < SA_STAGES; ++s) {
      umma::mbar_init(&S.full_b[s], 1);
      umma::mbar_init(&S.empty_b[s], SA_ISSUERS);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(&S.full_acc[b], SA_ISSUERS);
      umma::mbar_init(&S.empty_acc[b], 128);
    }
    umma::mbar_init(&S.mma_done, SA_ISSUERS);
    umma::fence_mbarrier_init();
    S.bad = 0;
    S.issued = 0;
    S.landed = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(&S.tmem, SA_TMEM_COLS);
    umma::tmem_relinquish();
  }
  // A: Z of the CTA's atoms over the window's nz, hi/lo
  for (int e = tid; e < SA_M * nzw; e += SA_THREADS) {
    const int r = e / nzw, z = e % nzw;
    const int a = blockIdx.x * SA_M + r;
    float sn = 0.f, cs = 0.f;
    if (a < n) sa_phase((int32_t)((uint32_t)(zb * nzw + z) * (uint32_t)F[a].z), &sn, &cs);
    __half rh, rl, ih, il;
    sa_split(cs, rh, rl);
    sa_split(sn, ih, il);
    const uint32_t off = umma::kmajor_offset(r, 2 * z, KA);
    *reinterpret_cast<__half2*>(A_hi + off) = __halves2half2(rh, ih);
    *reinterpret_cast<__half2*>(A_lo + off) = __halves2half2(rl, il);
  }
  umma::fence_proxy_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = S.tmem;

  if (warp == 4) {
    // ---- producer: chunk blobs in tile order through the ring
    if (lane == 0) {
      int g = 0;
      bool ok = true;
      for (int ti = 0; ti < n_list_tiles && ok; ++ti) {
        const int t = tile_list[ti];
        const int nq = tiles[t].n / 16;
        for (int q = 0; q < nq; ++q, ++g) {
          const int s = g % SA_STAGES;
          if (S.bad || !umma::mbar_wait(&S.empty_b[s], ((g / SA_STAGES) & 1) ^ 1, SA_WAIT)) {
            ok = false;
            break;
          }
          umma::mbar_expect_tx(&S.full_b[s], SA_BSTAGE);
          umma::bulk_g2s(B + (size_t)s * SA_BSTAGE, Bf + (size_t)(tile_chunk0[t] + q) * SA_BSTAGE, SA_BSTAGE,
                         &S.full_b[s]);
        }
      }
      if (!ok) S.bad = 1;
      S.issued = g;
    }
  } else if (warp == 5 || warp == 6) {
    // ---- MMA issuers: D[atom][row] per tile, warp 5 for T and warp 6 for T'
    // (separate accumulators, the same chunk stages: each stage and each
    // accumulator pair is released once both issuers' MMAs on it complete)
    const int which = warp - 5;
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_f16_f32(SA_M, SA_N);
      const uint32_t a_sbo = (uint32_t)(KA / 8) * 128, b_sbo = (SA_KC / 8) * 128;
      // descriptors built once; other stages, parts and k-steps add constants
      // to the address field (byte address >> 4)
      const uint64_t a_hi = umma::smem_desc(umma::smem_addr(A_hi), 128, a_sbo);
      const uint64_t a_lo = umma::smem_desc(umma::smem_addr(A_lo), 128, a_sbo);
      const uint64_t b_desc0 = umma::smem_desc(umma::smem_addr(B), 128, b_sbo);
      int g = 0;
      bool ok = true;
      for (int ti = 0; ti < n_list_tiles && ok; ++ti) {
        const int t = tiles[tile_list[ti]].n / 16;  // chunks of this tile
        const int buf = ti & 1;
        if (S.bad || !umma::mbar_wait(&S.empty_acc[buf], ((ti >> 1) & 1) ^ 1, SA_WAIT)) {
          ok = false;
          break;
        }
        for (int q = 0; q < t; ++q, ++g) {
          const int s = g % SA_STAGES;
          if (!umma::mbar_wait(&S.full_b[s], (g / SA_STAGES) & 1, SA_WAIT)) {
            ok = false;
            break;
          }
          atomicMax(&S.landed, g + 1);
          umma::fence_after_sync();
          const uint64_t b0 = b_desc0 + (uint64_t)(s * (SA_BSTAGE >> 4));
          const uint64_t aq = (uint64_t)(4 * q * 8);  // K offset of chunk q: 4q core matrices of 128 B
          {
            const uint32_t d = tmem + (uint32_t)(buf * 256 + which * 128);
            const uint64_t bh = b0 + (uint64_t)(2 * which * (SA_BPART >> 4));
            const uint64_t bl = bh + (uint64_t)(SA_BPART >> 4);
            const uint64_t ap[3] = {a_hi + aq, a_lo + aq, a_hi + aq}, bp[3] = {bl, bh, bh};
#pragma unroll
            for (int pass = 0; pass < 3; ++pass)
#pragma unroll
              for (int ks = 0; ks < 2; ++ks)
                umma::mma_f16(d, ap[pass] + (uint64_t)(ks * 16), bp[pass] + (uint64_t)(ks * 16), idesc,
                              (q == 0 && pass == 0 && ks == 0) ? 0u : 1u);
          }
          umma::mma_commit(&S.empty_b[s]);
        }
        if (!ok) break;
        umma::mma_commit(&S.full_acc[buf]);
      }
      if (!ok) S.bad = 1;
      umma::mma_commit(&S.mma_done);
      if (!umma::mbar_wait(&S.mma_done, 0, SA_WAIT)) S.bad = 1;
    }
  } else {
    // ---- epilogue: one atom per thread (TMEM lane)
    const uint32_t lanes = (uint32_t)(32 * warp) << 16;
    const int atom = blockIdx.x * SA_M + 32 * warp + lane;
    const int4 qa = atom < n ? F[atom] : make_int4(0, 0, 0, 0);
    float acc[3] = {0.f, 0.f, 0.f}, cmp[3] = {0.f, 0.f, 0.f};
    bool ok = true;
    for (int ti = 0; ti < n_list_tiles; ++ti) {
      const TcTile T = tiles[tile_list[ti]];
      const int buf = ti & 1;
      bool go = true;
      if (lane == 0) go = !S.bad && umma::mbar_wait(&S.full_acc[buf], (ti >> 1) & 1, SA_WAIT);
      if (!__shfl_sync(0xffffffffu, go ? 1 : 0, 0)) {
        ok = false;
        break;
      }
      umma::fence_after_sync();
      float xr[8], xi[8], yr[8], yi[8];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        sa_phase((int32_t)((uint32_t)(T.nx0 + a) * (uint32_t)qa.x), &xi[a], &xr[a]);
        sa_phase((int32_t)((uint32_t)(T.ny0 + a) * (uint32_t)qa.y), &yi[a], &yr[a]);
      }
      float px = 0.f, py = 0.f, pz = 0.f;
#pragma unroll
      for (int cb = 0; cb < SA_N; cb += 16) {
        uint32_t vt[16], vz[16];
        umma::tmem_ld_32x32b_x16(tmem + lanes + (uint32_t)(buf * 256 + cb), vt);
        umma::tmem_ld_32x32b_x16(tmem + lanes + (uint32_t)(buf * 256 + 128 + cb), vz);
        umma::tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int m = cb / 2 + i;  // complex row: nx = nx0 + m % 8, ny = ny0 + m / 8
          const float wr = fmaf(xr[m & 7], yr[m >> 3], -xi[m & 7] * yi[m >> 3]);
          const float wi = fmaf(xr[m & 7], yi[m >> 3], xi[m & 7] * yr[m >> 3]);
          const float v = fmaf(wr, __uint_as_float(vt[2 * i + 1]), wi * __uint_as_float(vt[2 * i]));
          const float vp = fmaf(wr, __uint_as_float(vz[2 * i + 1]), wi * __uint_as_float(vz[2 * i]));
          px = fmaf((float)(T.nx0 + (m & 7)), v, px);
          py = fmaf((float)(T.ny0 + (m >> 3)), v, py);
          pz += vp;
        }
      }
      umma::fence_before_sync();
      umma::mbar_arrive(&S.empty_acc[buf]);
      const float part[3] = {px * inv_c, py * inv_c, pz * inv_cz};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float y = __fsub_rn(part[d], cmp[d]), t = __fadd_rn(acc[d], y);
        cmp[d] = __fsub_rn(__fsub_rn(t, acc[d]), y);
        acc[d] = t;
      }
    }
    if (!ok) S.bad = 1;
    if (ok && atom < n) {
      float* gp = grad + ((int64_t)f * n + atom) * 3;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float v = -scale * __fsub_rn(acc[d], cmp[d]);
        gp[d] = accumulate ? gp[d] + v : v;
      }
    }
  }

  __syncthreads();
  if (S.bad) {
    if (tid == 32 * 4)
      for (int g = S.landed; g < S.issued; ++g)
        umma::mbar_wait(&S.full_b[g % SA_STAGES], (g / SA_STAGES) & 1, SA_WAIT);
    if (tid == 0) atomicExch(err, 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, SA_TMEM_COLS);
  }
}

size_t sa_smem_bytes(int32_t nzw) {
  const size_t a = 2 * (size_t)SA_M * 2 * nzw * 2;
  return ((a + 1023) & ~(size_t)1023) + SA_STAGES * SA_BSTAGE + sizeof(SaBars) + 1024;
}

// Gradient of sum_s w_s S_raw[s] for a lattice density on the tensor cores.
// fx: fixed-point phases [F][n]; u: per-vector weights (2 w_s / H_s); rho the
// density's table; grad [F][n][3] on the device.
void sk_adjoint_tc_run(amdat_ctx* ctx, const TcPlan& P, const int4* fx, int32_t n, int32_t F,
                       const float2* rho, int32_t n_k, const float* d_u, float max_u, float period,
                       float* grad) {
  if (n == 0 || P.n_tiles == 0) return;
  AMDAT_REQUIRE(sa_smem_bytes(P.nzw) <= 232448, "nz window too wide for the tensor-core adjoint");
  // chunks in tile order; tile lists per nz window
  std::vector<int32_t> chunk_tile, chunk_q, tile_chunk0(P.n_tiles);
  std::vector<std::vector<int32_t>> by_zb(P.n_zblk);
  for (int t = 0; t < P.n_tiles; ++t) {
    const TcTile& T = P.host_tiles[t];
    tile_chunk0[t] = (int32_t)chunk_tile.size();
    for (int q = 0; q < T.n / 16; ++q) {
      chunk_tile.push_back(t);
      chunk_q.push_back(q);
    }
    by_zb[T.zblk].push_back(t);
  }
  const int32_t n_chunks = (int32_t)chunk_tile.size();
  // FP16 range: |c| <= max_u * n; keep the scaled values below 2^14
  const double bound = std::max(1e-30, (double)max_u * (double)n);
  const int e_c = (int)std::floor(std::log2(16384.0 / bound));
  const int e_z = e_c - (int)std::ceil(std::log2((double)P.nmax + 1.0));
  const float scale_c = (float)std::ldexp(1.0, e_c), scale_cz = (float)std::ldexp(1.0, e_z);
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t o = 0;
  const size_t o_ct = o; o = align(o + (size_t)n_chunks * 4);
  const size_t o_cq = o; o = align(o + (size_t)n_chunks * 4);
  const size_t o_t0 = o; o = align(o + (size_t)P.n_tiles * 4);
  const size_t o_tl = o; o = align(o + (size_t)P.n_tiles * 4);
  const size_t o_err = o; o = align(o + 4);
  const size_t o_blob = o; o = align(o + (size_t)F * n_chunks * SA_BSTAGE);
  unsigned char* base = ctx->scratch2.reserve(o);
  cudaStream_t st = ctx->stream;
  std::vector<int32_t> tl;
  for (auto& v : by_zb) tl.insert(tl.end(), v.begin(), v.end());
  AMDAT_CUDA(cudaMemcpyAsync(base + o_ct, chunk_tile.data(), (size_t)n_chunks * 4, cudaMemcpyHostToDevice, st));
  AMDAT_CUDA(cudaMemcpyAsync(base + o_cq, chunk_q.data(), (size_t)n_chunks * 4, cudaMemcpyHostToDevice, st));
  AMDAT_CUDA(cudaMemcpyAsync(base + o_t0, tile_chunk0.data(), (size_t)P.n_tiles * 4, cudaMemcpyHostToDevice, st));
  AMDAT_CUDA(cudaMemcpyAsync(base + o_tl, tl.data(), tl.size() * 4, cudaMemcpyHostToDevice, st));
  AMDAT_CUDA(cudaMemsetAsync(base + o_err, 0, 4, st));
  sa_blob_kernel<<<dim3((unsigned)n_chunks, (unsigned)F), 256, 0, st>>>(
      rho, n_k, d_u, P.tiles.ptr, P.entry_k.ptr, (const int32_t*)(base + o_ct), (const int32_t*)(base + o_cq),
      n_chunks, P.nzw, scale_c, scale_cz, base + o_blob);
  check_launch("sa_blob_kernel");
  count_launch(ctx);
  const size_t shm = sa_smem_bytes(P.nzw);
  AMDAT_CUDA(cudaFuncSetAttribute(sk_adjoint_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  const float sc = (float)(6.283185307179586476925286766559 / (double)period);
  size_t first = 0;
  for (int zb = 0; zb < P.n_zblk; ++zb) {
    const size_t cnt = by_zb[zb].size();
    if (!cnt) continue;
    KernelTimer kt(ctx, "sk_adjoint_tc_kernel");
    sk_adjoint_tc_kernel<<<dim3((unsigned)ceil_div(n, SA_M), (unsigned)F), SA_THREADS, shm, st>>>(
        fx, n, zb, P.nzw, P.tiles.ptr, (const int32_t*)(base + o_tl) + first, (int32_t)cnt,
        (const int32_t*)(base + o_t0), base + o_blob, n_chunks, 1.0f / scale_c, 1.0f / scale_cz, sc,
        first > 0 ? 1 : 0, grad, (int*)(base + o_err));
    check_launch("sk_adjoint_tc_kernel");
    count_launch(ctx);
    first += cnt;
  }
  int h_err = 0;
  AMDAT_CUDA(cudaMemcpyAsync(&h_err, base + o_err, 4, cudaMemcpyDeviceToHost, st));
  AMDAT_CUDA(cudaStreamSynchronize(st));
  if (h_err) throw Error(AMDAT_ERR_TIMEOUT, "tensor-core S(k) adjoint: a bounded wait timed out");
}

}  // namespace amdat
