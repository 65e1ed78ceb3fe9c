// Tensor-core (tcgen05) Fourier densities over the whole half-space lattice.
//
// rho[(nx,ny), nz] = sum_j W_j(nx,ny) Z_j(nz), W = X(nx) Y(ny), is a complex
// GEMM with the atoms as the reduction axis.  As a real GEMM per tile:
//   A (128 x 2J): rows 0..63   = [Wr, -Wi] of 64 (nx,ny) rows (8 nx x 8 ny),
//                 rows 64..127 = [Wi,  Wr]           (k = 2j, 2j+1 per atom j)
//   B ( 64 x 2J): [Zr, Zi] for 64 consecutive nz
//   D = A B^T  (128 x 64): rows 0..63 = Re rho, rows 64..127 = Im rho.
// Operands are FP16 split into hi + lo parts (x = hi + lo to ~2^-22), and each
// chunk runs three tcgen05.mma passes, hi*hi + hi*lo + lo*hi, accumulating in
// FP32 tensor memory; after every TC_GROUP chunks (64 atoms) the accumulator
// is drained into Kahan-compensated FP32 registers (the tensor core's FP32
// accumulation drops low bits as the accumulator grows, so it never spans more
// than 64 atoms), double-buffered so the next MMAs overlap the drain.  The phases are the exact fixed-point phases of
// the FP32 kernels (fraction of the box in units of 2^-31 turns).
//
// Per frame batch, zgen_kernel precomputes the B operands (Z hi/lo in the
// K-major core-matrix layout, one 16 KB blob per (frame, nz block, 32-atom
// chunk)); the main kernel streams them with 1-D bulk copies (cp.async.bulk)
// into a two-stage shared-memory ring and builds A from per-chunk X/Y phase
// tables.  One thread issues the MMAs; mbarriers order bulk copy -> MMA ->
// stage reuse and MMA -> tensor-memory drain; every wait is bounded and a
// timeout is reported through an error word.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "umma.cuh"

namespace amdat {

constexpr int TC_J = 32;                      // atoms per chunk
constexpr int TC_K = 2 * TC_J;                // real K per chunk
constexpr int TC_ROWS = 64;                   // complex rows (8 nx x 8 ny)
constexpr int TC_NZ = 64;                     // nz columns per tile (MMA N)
constexpr int TC_M = 2 * TC_ROWS;             // MMA M = 128
constexpr int TC_THREADS = 256;
constexpr uint32_t TC_A_BYTES = TC_M * TC_K * 2;    // 16 KB (one of hi / lo)
constexpr uint32_t TC_B_BYTES = TC_NZ * TC_K * 2;   // 8 KB (one of hi / lo)
constexpr uint32_t TC_BLOB = 2 * TC_B_BYTES;        // Z hi + lo per (frame, nz block, chunk)
constexpr uint32_t TC_WAIT = 1u << 22;              // mbarrier polls (~0.5 s bound)
constexpr int TC_GROUP = 2;                          // chunks per tensor-memory accumulation

struct TcTile {
  int32_t nx0, ny0, zblk, entry0;  // entry map: TC_ROWS * TC_NZ ints from entry0
};

struct TcSmem {
  unsigned char a[2][2][TC_A_BYTES];  // [stage][hi|lo]
  unsigned char b[2][TC_BLOB];        // [stage] hi then lo
  float2 xy[2][TC_J * 16];            // [stage][atom*16 + swizzled(8 X then 8 Y)]
  uint64_t mbar_tma[2];
  uint64_t mbar_mma[2];
  uint32_t tmem;
  int bad;
};

__device__ __forceinline__ void tc_split(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(__fsub_rn(x, __half2float(hi)));
}

__device__ __forceinline__ void tc_phase(int32_t ph, float* s, float* c) {
  sincospif(__fmul_rn((float)ph, 9.313225746154785e-10f), s, c);  // ph * 2^-30 * pi
}

// Z operands of one frame batch: blob (f, zblk, chunk) = [hi 8 KB][lo 8 KB],
// each a 64 (nz) x 64 (k) K-major tile; k = 2j -> Re Z_j, 2j+1 -> Im Z_j
__global__ void __launch_bounds__(256)
    zgen_kernel(const int4* __restrict__ fx, int32_t n_list, int32_t n_chunks, int32_t n_zblk,
                unsigned char* __restrict__ zbuf) {
  const int blob = blockIdx.x;
  const int c = blob % n_chunks;
  const int zb = (blob / n_chunks) % n_zblk;
  const int f = blob / (n_chunks * n_zblk);
  unsigned char* hi = zbuf + (size_t)blob * TC_BLOB;
  unsigned char* lo = hi + TC_B_BYTES;
  const int4* F = fx + (int64_t)f * n_list;
  for (int e = threadIdx.x; e < TC_NZ * TC_J; e += blockDim.x) {
    const int col = e % TC_NZ, j = e / TC_NZ;
    const int a = c * TC_J + j;
    float s = 0.f, co = 0.f;
    if (a < n_list) {
      const int32_t nz = zb * TC_NZ + col;
      tc_phase((int32_t)((uint32_t)nz * (uint32_t)F[a].z), &s, &co);
    }
    __half rh, rl, ih, il;
    tc_split(co, rh, rl);
    tc_split(s, ih, il);
    const uint32_t off = umma::kmajor_offset(col, 2 * j, TC_K);
    *reinterpret_cast<__half2*>(hi + off) = __halves2half2(rh, ih);
    *reinterpret_cast<__half2*>(lo + off) = __halves2half2(rl, il);
  }
}

// X/Y table slot of (atom j, entry m): rotating the 16 entries by 4*(j%4)
// spreads a warp's reads (8 rows x 4 atoms) over all banks
__device__ __forceinline__ int xy_slot(int j, int m) { return j * 16 + ((m + 4 * (j & 3)) & 15); }

struct KCf {
  float s, c;
};

__global__ void __launch_bounds__(TC_THREADS, 2)
    rhok_tc_kernel(const int4* __restrict__ fx, int32_t n_list, int32_t n_chunks, int32_t n_zblk,
                   const TcTile* __restrict__ tiles, const int32_t* __restrict__ entry_k,
                   const unsigned char* __restrict__ zbuf, int32_t frame0, int32_t n_k,
                   float2* __restrict__ rho, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
  const TcTile T = tiles[blockIdx.x];
  const int fl = blockIdx.y;  // frame within the batch
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int4* F = fx + (int64_t)fl * n_list;
  const unsigned char* Z = zbuf + ((size_t)fl * n_zblk + T.zblk) * (size_t)n_chunks * TC_BLOB;

  if (tid == 0) {
    umma::mbar_init(&S.mbar_tma[0], 1);
    umma::mbar_init(&S.mbar_tma[1], 1);
    umma::mbar_init(&S.mbar_mma[0], 1);
    umma::mbar_init(&S.mbar_mma[1], 1);
    umma::fence_mbarrier_init();
    S.bad = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(&S.tmem, 2 * TC_NZ);  // two 64-column accumulators
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = S.tmem;
  // this thread's accumulator slice: TMEM lanes 32*(warp%4)+lane, columns 32*(warp/4)..+31
  const uint32_t t_lane = (uint32_t)(32 * (warp & 3)) << 16;
  const uint32_t t_col = (uint32_t)(32 * (warp >> 2));
  KCf acc[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) acc[i] = KCf{0.f, 0.f};
  const uint32_t idesc = umma::idesc_f16_f32(TC_M, TC_NZ);
  constexpr uint32_t LBO = 128, SBO = (TC_K / 8) * 128;

  auto drain = [&](int buf) {
    umma::fence_after_sync();
    uint32_t r[32];
    umma::tmem_ld_32x32b_x32(tmem + t_lane + (uint32_t)(buf * TC_NZ) + t_col, r);
    umma::tmem_ld_wait();
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const float v = __uint_as_float(r[i]);
      const float y = __fsub_rn(v, acc[i].c);
      const float t = __fadd_rn(acc[i].s, y);
      acc[i].c = __fsub_rn(__fsub_rn(t, acc[i].s), y);
      acc[i].s = t;
    }
    umma::fence_before_sync();
  };

  // X (8) and Y (8) phase tables of chunk cc's atoms, into xy[cc & 1]
  auto build_xy = [&](int cc) {
    for (int e = tid; e < TC_J * 16; e += TC_THREADS) {
      const int j = e >> 4, m = e & 15;
      const int a = cc * TC_J + j;
      float sn = 0.f, cs = 0.f;
      if (a < n_list) {
        const int4 q = F[a];
        const int32_t ph = m < 8 ? (int32_t)((uint32_t)(T.nx0 + m) * (uint32_t)q.x)
                                 : (int32_t)((uint32_t)(T.ny0 + m - 8) * (uint32_t)q.y);
        tc_phase(ph, &sn, &cs);
      }
      S.xy[cc & 1][xy_slot(j, m)] = make_float2(cs, sn);
    }
  };
  // prologue: Z operands of chunks 0 and 1 in flight, X/Y of chunk 0
  if (tid == 0)
    for (int cc = 0; cc < 2 && cc < n_chunks; ++cc) {
      umma::mbar_expect_tx(&S.mbar_tma[cc], TC_BLOB);
      umma::bulk_g2s(S.b[cc], Z + (size_t)cc * TC_BLOB, TC_BLOB, &S.mbar_tma[cc]);
    }
  build_xy(0);
  __syncthreads();

  // Pipeline per chunk c (stage s = c & 1, accumulator s):
  //   all threads: A(c) into stage s, X/Y of chunk c+1        | MMA(c-1) runs
  //   thread 0:    wait Z(c); issue MMA(c); wait MMA(c-1);
  //                bulk-copy Z(c+1) into stage s^1 (now free)
  //   all threads: drain accumulator s^1 (chunk c-1)           | MMA(c) runs
  int c = 0;
  for (; c < n_chunks; ++c) {
    const int s = c & 1;
    // A operand: lane = (row % 8) * 4 + (atom % 4), conflict-free 4-byte stores
#pragma unroll 2
    for (int it = 0; it < 8; ++it) {
      const int combo = warp * 8 + it;  // 0..63
      const int rg = combo >> 3, jg = combo & 7;
      const int r = rg * 8 + (lane >> 2);   // complex row: nx = r % 8, ny = r / 8
      const int j = jg * 4 + (lane & 3);
      const float2 x = S.xy[s][xy_slot(j, r & 7)], y = S.xy[s][xy_slot(j, 8 + (r >> 3))];
      const float wr = fmaf(x.x, y.x, -x.y * y.y), wi = fmaf(x.x, y.y, x.y * y.x);
      // hi = fp16(w), lo = fp16(w - hi), both as (re, im) half2 pairs
      const __half2 hi = __floats2half2_rn(wr, wi);
      const float2 hb = __half22float2(hi);
      const __half2 lo = __floats2half2_rn(__fsub_rn(wr, hb.x), __fsub_rn(wi, hb.y));
      const uint32_t h = *reinterpret_cast<const uint32_t*>(&hi);
      const uint32_t l = *reinterpret_cast<const uint32_t*>(&lo);
      const uint32_t o_re = umma::kmajor_offset(r, 2 * j, TC_K);
      const uint32_t o_im = umma::kmajor_offset(TC_ROWS + r, 2 * j, TC_K);
      // real rows (Wr, -Wi): flip the sign of the high half; imaginary rows (Wi, Wr): swap halves
      *reinterpret_cast<uint32_t*>(S.a[s][0] + o_re) = h ^ 0x80000000u;
      *reinterpret_cast<uint32_t*>(S.a[s][1] + o_re) = l ^ 0x80000000u;
      *reinterpret_cast<uint32_t*>(S.a[s][0] + o_im) = __byte_perm(h, 0, 0x1032);
      *reinterpret_cast<uint32_t*>(S.a[s][1] + o_im) = __byte_perm(l, 0, 0x1032);
    }
    if (c + 1 < n_chunks) build_xy(c + 1);
    umma::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      if (!umma::mbar_wait(&S.mbar_tma[s], (c >> 1) & 1, TC_WAIT)) {
        S.bad = 1;
      } else {
        umma::fence_after_sync();
        const uint32_t d = tmem + (uint32_t)(((c / TC_GROUP) & 1) * TC_NZ);
        const uint32_t a_hi = umma::smem_addr(S.a[s][0]), a_lo = umma::smem_addr(S.a[s][1]);
        const uint32_t b_hi = umma::smem_addr(S.b[s]), b_lo = b_hi + TC_B_BYTES;
        // small cross terms first, then hi*hi, so the accumulator is still small
        // while the 2^-11-sized terms are added
        const uint32_t pa[3] = {a_hi, a_lo, a_hi}, pb[3] = {b_lo, b_hi, b_hi};
#pragma unroll
        for (int pass = 0; pass < 3; ++pass)
#pragma unroll
          for (int ks = 0; ks < TC_K / 16; ++ks)
            umma::mma_f16(d, umma::smem_desc(pa[pass] + ks * 256, LBO, SBO),
                          umma::smem_desc(pb[pass] + ks * 256, LBO, SBO), idesc,
                          (c % TC_GROUP == 0 && pass == 0 && ks == 0) ? 0u : 1u);
        umma::mma_commit(&S.mbar_mma[s]);
      }
      if (!S.bad && c >= 1) {
        if (!umma::mbar_wait(&S.mbar_mma[s ^ 1], ((c - 1) >> 1) & 1, TC_WAIT)) {
          S.bad = 1;
        } else if (c + 1 < n_chunks) {
          umma::mbar_expect_tx(&S.mbar_tma[s ^ 1], TC_BLOB);
          umma::bulk_g2s(S.b[s ^ 1], Z + (size_t)(c + 1) * TC_BLOB, TC_BLOB, &S.mbar_tma[s ^ 1]);
        }
      }
    }
    __syncthreads();
    if (S.bad) break;
    // a new accumulation group started: drain the previous group's buffer
    if (c % TC_GROUP == 0 && c >= 1) drain(((c / TC_GROUP) & 1) ^ 1);
  }
  __syncthreads();
  const int last = c - 1;
  if (!S.bad && last >= 0) {
    if (tid == 0 && !umma::mbar_wait(&S.mbar_mma[last & 1], (last >> 1) & 1, TC_WAIT)) S.bad = 1;
    __syncthreads();
    if (!S.bad) drain((last / TC_GROUP) & 1);
  }
  __syncthreads();
  if (!S.bad) {
    // stage D through shared memory (reusing the A buffers) to pair Re / Im rows
    constexpr int DP = TC_NZ + 1;  // padded row: lanes of a warp hit different banks
    float* D = reinterpret_cast<float*>(S.a[0][0]);  // [128][DP]: 33 KB from the start of the A buffers
    const int row = 32 * (warp & 3) + lane;
#pragma unroll
    for (int i = 0; i < 32; ++i) D[row * DP + t_col + i] = __fsub_rn(acc[i].s, acc[i].c);
    __syncthreads();
    const int32_t* E = entry_k + T.entry0;
    float2* out = rho + (int64_t)(frame0 + fl) * n_k;
    for (int e = tid; e < TC_ROWS * TC_NZ; e += TC_THREADS) {
      const int k = E[e];
      if (k >= 0) {
        const int r = e / TC_NZ, col = e % TC_NZ;
        out[k] = make_float2(D[r * DP + col], D[(TC_ROWS + r) * DP + col]);
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 2 * TC_NZ);
  }
}

// ---------------------------------------------------------------------------
// host: tile plan over the shell-sorted vector list, launches per frame batch
// ---------------------------------------------------------------------------
struct TcPlan {
  DevBuf<TcTile> tiles;
  DevBuf<int32_t> entry_k;
  int32_t n_tiles = 0, n_zblk = 0;
};

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
  std::vector<TcTile> tiles;
  std::vector<int32_t> entries;
  const int n_zblk = (nmax + TC_NZ) / TC_NZ;
  for (int x0 = -nmax; x0 <= nmax; x0 += 8)
    for (int y0 = -nmax; y0 <= nmax; y0 += 8)
      for (int zb = 0; zb < n_zblk; ++zb) {
        std::vector<int32_t> e(TC_ROWS * TC_NZ, -1);
        bool any = false;
        for (int r = 0; r < TC_ROWS; ++r)
          for (int c = 0; c < TC_NZ; ++c) {
            const int nx = x0 + (r & 7), ny = y0 + (r >> 3), nz = zb * TC_NZ + c;
            if (nx > nmax || ny > nmax || nz > nmax) continue;
            const int k = index[((size_t)(nx + nmax) * W + (ny + nmax)) * H + nz];
            if (k >= 0) {
              e[r * TC_NZ + c] = k;
              any = true;
            }
          }
        if (!any) continue;
        tiles.push_back(TcTile{x0, y0, zb, (int32_t)entries.size()});
        entries.insert(entries.end(), e.begin(), e.end());
      }
  auto* p = new TcPlan();
  p->n_tiles = (int32_t)tiles.size();
  p->n_zblk = n_zblk;
  p->tiles.reserve(std::max<size_t>(tiles.size(), 1));
  p->entry_k.reserve(std::max<size_t>(entries.size(), 1));
  if (!tiles.empty()) {
    AMDAT_CUDA(cudaMemcpy(p->tiles.ptr, tiles.data(), tiles.size() * sizeof(TcTile), cudaMemcpyHostToDevice));
    AMDAT_CUDA(cudaMemcpy(p->entry_k.ptr, entries.data(), entries.size() * 4, cudaMemcpyHostToDevice));
  }
  return p;
}

void tc_plan_free(TcPlan* p) { delete p; }

// rho[f][k] for frames 0..n_frames-1 of fx ([n_frames][n_list] fixed-point phases)
void rhok_tc_run(amdat_ctx* ctx, const TcPlan& P, const int4* fx, int32_t n_list, int32_t n_frames,
                 int32_t n_k, float2* rho) {
  if (P.n_tiles == 0 || n_list == 0 || n_frames == 0) return;
  const int32_t n_chunks = (int32_t)ceil_div(n_list, TC_J);
  const size_t per_frame = (size_t)P.n_zblk * n_chunks * TC_BLOB;
  // frame batches bound the Z-operand buffer to ~1 GB
  const int32_t batch = (int32_t)std::max<size_t>(1, std::min<size_t>(n_frames, (size_t)(1u << 30) / per_frame));
  unsigned char* zbuf = ctx->scratch.reserve(per_frame * batch + 256);
  int* d_err = (int*)(zbuf + per_frame * batch);
  AMDAT_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  const size_t shm = sizeof(TcSmem) + 1024;
  AMDAT_CUDA(cudaFuncSetAttribute(rhok_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
  for (int32_t f0 = 0; f0 < n_frames; f0 += batch) {
    const int32_t nb = std::min(batch, n_frames - f0);
    zgen_kernel<<<(unsigned)(nb * P.n_zblk * n_chunks), 256, 0, ctx->stream>>>(
        fx + (int64_t)f0 * n_list, n_list, n_chunks, P.n_zblk, zbuf);
    check_launch("zgen_kernel");
    count_launch(ctx);
    KernelTimer kt(ctx, "rhok_tc_kernel");
    dim3 grid((unsigned)P.n_tiles, (unsigned)nb);
    rhok_tc_kernel<<<grid, TC_THREADS, shm, ctx->stream>>>(fx + (int64_t)f0 * n_list, n_list, n_chunks,
                                                          P.n_zblk, P.tiles.ptr, P.entry_k.ptr, zbuf,
                                                          f0, n_k, rho, d_err);
    check_launch("rhok_tc_kernel");
    count_launch(ctx);
  }
  int h_err = 0;
  AMDAT_CUDA(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h_err) throw Error(AMDAT_ERR_TIMEOUT, "tensor-core rho_k: a bounded wait timed out");
}

}  // namespace amdat
