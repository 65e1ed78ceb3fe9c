// Fourier densities rho(k,t) = sum_j exp(i k.r_j(t)), k = 2 pi n / L, on the GPU.
//
// Replaces Wave_Density::analyze / listkernel (src/wave_density.cpp:313-365)
// and the density part of Structure_Factor::listkernel
// (src/structure_factor.cpp:293-320), which evaluate cosf/sinf of an FP32 dot
// product k.r per atom and vector.
//
// Phases are exact: each wrapped coordinate is converted once per frame (in
// FP64) to a fixed-point fraction of the box, f = r/L mod 1 in units of 2^-31
// turns (int32).  The phase of an integer lattice vector n is then the int32
// combination nx*fx + ny*fy + nz*fz, exact modulo whole turns (int32 wraps at
// two turns), and only the final conversion to FP32 rounds (<= 2e-7 rad)
// before sincospif.  (An FP32 k.r as in the reference loses ~1e-4 rad once
// |k.r| ~ 1000.)
//
// Kernels:
//   rhok_list_kernel     any vector list (e.g. the reference's q-vector
//                        shells): a block owns 1024 vectors of one frame and
//                        streams the frame's atoms through shared memory.
//   rhok_lattice_kernel  every half-space lattice vector with |n| <= R,
//                        factorised as rho[(nx,ny), nz] = sum_j W_j(nx,ny) Z_j(nz)
//                        with W = X(nx) Y(ny): a complex outer-product
//                        accumulation over atoms on the FP32 pipes.  A tile is
//                        16 nx x 8 ny rows x 32 nz columns; per chunk of 32
//                        atoms the block builds X, Y, Z by sincospif and W by
//                        products in shared memory, then every thread
//                        accumulates a 4x4 block of outputs (64 FMA per atom).
//   rhok_plain_kernel    FP64 direct sum (the plain path).
// FP32 accumulators are folded into Kahan-compensated sums every 128 atoms.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>

#include "engine.h"
#include "tc_tiles.h"

namespace amdat {

void ensure_fp64(amdat_ctx* ctx);

struct ListView {
  int32_t n;
  int32_t first;
  const int32_t* idx;
};

static ListView view(const ListEntry& e) {
  return ListView{e.n, e.first, e.contiguous ? nullptr : e.idx.ptr};
}

// wrapped coordinate -> int32 fraction of a turn (units of 2^-31), in FP64
__global__ void fixed_turns_kernel(const float* __restrict__ w, int64_t n_pad, int32_t n_frames,
                                   const int32_t* __restrict__ frames, ListView lst,
                                   double inv_period, int4* __restrict__ out) {
  const int64_t total = (int64_t)n_frames * lst.n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int f = (int)(i / lst.n), a = (int)(i % lst.n);
    const int atom = lst.idx ? lst.idx[a] : lst.first + a;
    const float* P = w + (int64_t)frames[f] * 3 * n_pad;
    int32_t q[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double t = (double)P[c * n_pad + atom] * inv_period;
      t -= rint(t);
      q[c] = (int32_t)llrint(t * 2147483648.0);
    }
    out[i] = make_int4(q[0], q[1], q[2], 0);
  }
}

__device__ __forceinline__ void phase_sincos(int32_t ph, float* s, float* c) {
  sincospif(__fmul_rn((float)ph, 9.313225746154785e-10f), s, c);  // angle = ph * 2^-30 * pi
}

struct KC {  // compensated complex sum, value = s - c
  float sr, si, cr, ci;
};
__device__ __forceinline__ void kc_add(KC& k, float re, float im) {
  float y = __fsub_rn(re, k.cr), t = __fadd_rn(k.sr, y);
  k.cr = __fsub_rn(__fsub_rn(t, k.sr), y);
  k.sr = t;
  y = __fsub_rn(im, k.ci);
  t = __fadd_rn(k.si, y);
  k.ci = __fsub_rn(__fsub_rn(t, k.si), y);
  k.si = t;
}

// ---------------------------------------------------------------------------
// list mode
// ---------------------------------------------------------------------------
constexpr int RL_THREADS = 256;
constexpr int RL_KPT = 4;                       // vectors per thread
constexpr int RL_TILE = RL_THREADS * RL_KPT;    // vectors per block
constexpr int RL_ATOMS = 512;                   // atoms staged per step

__global__ void __launch_bounds__(RL_THREADS)
    rhok_list_kernel(const int4* __restrict__ fx, int32_t n_list, const int4* __restrict__ kv,
                     int32_t n_k, float2* __restrict__ rho) {
  __shared__ int4 s_at[RL_ATOMS];
  const int f = blockIdx.y;
  const int k0 = blockIdx.x * RL_TILE;
  int4 n[RL_KPT];
  KC acc[RL_KPT];
  float pr[RL_KPT], pi[RL_KPT];
#pragma unroll
  for (int j = 0; j < RL_KPT; ++j) {
    const int k = k0 + j * RL_THREADS + threadIdx.x;
    n[j] = k < n_k ? kv[k] : make_int4(0, 0, 0, 0);
    acc[j] = KC{0.f, 0.f, 0.f, 0.f};
    pr[j] = pi[j] = 0.f;
  }
  const int4* F = fx + (int64_t)f * n_list;
  int since_fold = 0;
  for (int a0 = 0; a0 < n_list; a0 += RL_ATOMS) {
    const int na = min(RL_ATOMS, n_list - a0);
    __syncthreads();
    for (int i = threadIdx.x; i < na; i += RL_THREADS) s_at[i] = F[a0 + i];
    __syncthreads();
    for (int a = 0; a < na; ++a) {
      const int4 q = s_at[a];
#pragma unroll
      for (int j = 0; j < RL_KPT; ++j) {
        const int32_t ph = (int32_t)((uint32_t)n[j].x * (uint32_t)q.x +
                                     (uint32_t)n[j].y * (uint32_t)q.y +
                                     (uint32_t)n[j].z * (uint32_t)q.z);
        float s, c;
        phase_sincos(ph, &s, &c);
        pr[j] += c;
        pi[j] += s;
      }
      if (++since_fold == 128) {
#pragma unroll
        for (int j = 0; j < RL_KPT; ++j) {
          kc_add(acc[j], pr[j], pi[j]);
          pr[j] = pi[j] = 0.f;
        }
        since_fold = 0;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < RL_KPT; ++j) {
    kc_add(acc[j], pr[j], pi[j]);
    const int k = k0 + j * RL_THREADS + threadIdx.x;
    if (k < n_k)
      rho[(int64_t)f * n_k + k] = make_float2(__fsub_rn(acc[j].sr, acc[j].cr),
                                              __fsub_rn(acc[j].si, acc[j].ci));
  }
}

// ---------------------------------------------------------------------------
// lattice mode
// ---------------------------------------------------------------------------
constexpr int LT_NX = 16, LT_NY = 8, LT_NZ = 32;
constexpr int LT_ROWS = LT_NX * LT_NY;  // 128
constexpr int LT_THREADS = 256;
constexpr int LT_A = 32;  // atoms per chunk
constexpr int LT_FOLD = 4;  // chunks between compensated folds

struct LatticeTile {
  int32_t nx0, ny0, nz0;
  int32_t entry0;  // first entry of this tile in the entry map (tile-major, LT_ROWS*LT_NZ)
};

__global__ void __launch_bounds__(LT_THREADS, 2)
    rhok_lattice_kernel(const int4* __restrict__ fx, int32_t n_list,
                        const LatticeTile* __restrict__ tiles,
                        const int32_t* __restrict__ entry_k, int32_t n_k,
                        float2* __restrict__ rho) {
  __shared__ __align__(16) float2 sW[LT_A][LT_ROWS];
  __shared__ __align__(16) float2 sZ[LT_A][LT_NZ];
  __shared__ float2 sX[LT_A][LT_NX];
  __shared__ float2 sY[LT_A][LT_NY];
  const LatticeTile T = tiles[blockIdx.x];
  const int f = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // warp covers 8 row-groups x 4 col-groups; a thread owns 4 rows x 4 cols
  const int rg = (warp & 3) * 8 + (lane & 7);  // 0..31
  const int cg = (warp >> 2) * 4 + (lane >> 3); // 0..7
  float ar[4][4], ai[4][4];
  KC acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      ar[r][c] = ai[r][c] = 0.f;
      acc[r][c] = KC{0.f, 0.f, 0.f, 0.f};
    }
  const int4* F = fx + (int64_t)f * n_list;
  int chunk = 0;
  for (int a0 = 0; a0 < n_list; a0 += LT_A, ++chunk) {
    __syncthreads();
    // X (16), Y (8), Z (32) phase tables for LT_A atoms: 56 * 32 = 1792 entries
    for (int e = tid; e < LT_A * (LT_NX + LT_NY + LT_NZ); e += LT_THREADS) {
      const int a = e / (LT_NX + LT_NY + LT_NZ), m = e % (LT_NX + LT_NY + LT_NZ);
      float s = 0.f, c = 0.f;
      if (a0 + a < n_list) {
        const int4 q = F[a0 + a];
        int32_t ph;
        if (m < LT_NX) ph = (int32_t)((uint32_t)(T.nx0 + m) * (uint32_t)q.x);
        else if (m < LT_NX + LT_NY) ph = (int32_t)((uint32_t)(T.ny0 + m - LT_NX) * (uint32_t)q.y);
        else ph = (int32_t)((uint32_t)(T.nz0 + m - LT_NX - LT_NY) * (uint32_t)q.z);
        phase_sincos(ph, &s, &c);
      }
      if (m < LT_NX) sX[a][m] = make_float2(c, s);
      else if (m < LT_NX + LT_NY) sY[a][m - LT_NX] = make_float2(c, s);
      else sZ[a][m - LT_NX - LT_NY] = make_float2(c, s);
    }
    __syncthreads();
    for (int e = tid; e < LT_A * LT_ROWS; e += LT_THREADS) {
      const int a = e / LT_ROWS, r = e % LT_ROWS;
      const float2 x = sX[a][r % LT_NX], y = sY[a][r / LT_NX];
      sW[a][r] = make_float2(fmaf(x.x, y.x, -x.y * y.y), fmaf(x.x, y.y, x.y * y.x));
    }
    __syncthreads();
#pragma unroll 4
    for (int a = 0; a < LT_A; ++a) {
      const float4 w01 = *reinterpret_cast<const float4*>(&sW[a][rg * 4]);
      const float4 w23 = *reinterpret_cast<const float4*>(&sW[a][rg * 4 + 2]);
      const float4 z01 = *reinterpret_cast<const float4*>(&sZ[a][cg * 4]);
      const float4 z23 = *reinterpret_cast<const float4*>(&sZ[a][cg * 4 + 2]);
      const float wr[4] = {w01.x, w01.z, w23.x, w23.z}, wi[4] = {w01.y, w01.w, w23.y, w23.w};
      const float zr[4] = {z01.x, z01.z, z23.x, z23.z}, zi[4] = {z01.y, z01.w, z23.y, z23.w};
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          ar[r][c] = fmaf(wr[r], zr[c], fmaf(-wi[r], zi[c], ar[r][c]));
          ai[r][c] = fmaf(wr[r], zi[c], fmaf(wi[r], zr[c], ai[r][c]));
        }
    }
    if ((chunk + 1) % LT_FOLD == 0) {
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          kc_add(acc[r][c], ar[r][c], ai[r][c]);
          ar[r][c] = ai[r][c] = 0.f;
        }
    }
  }
  const int32_t* E = entry_k + T.entry0;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      kc_add(acc[r][c], ar[r][c], ai[r][c]);
      const int row = rg * 4 + r, col = cg * 4 + c;
      const int k = E[row * LT_NZ + col];
      if (k >= 0)
        rho[(int64_t)f * n_k + k] = make_float2(__fsub_rn(acc[r][c].sr, acc[r][c].cr),
                                                __fsub_rn(acc[r][c].si, acc[r][c].ci));
    }
}

// ---------------------------------------------------------------------------
// plain FP64 path: one thread per (frame, vector), FP64 sincos
// ---------------------------------------------------------------------------
__global__ void rhok_plain_kernel(const double* __restrict__ w, int64_t n_pad,
                                  const int32_t* __restrict__ frames, ListView lst,
                                  const int4* __restrict__ kv, int32_t n_k, double two_pi_over_l,
                                  float2* __restrict__ rho) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = blockIdx.y;
  if (k >= n_k) return;
  const int4 n = kv[k];
  const double kx = two_pi_over_l * n.x, ky = two_pi_over_l * n.y, kz = two_pi_over_l * n.z;
  const double* P = w + (int64_t)frames[f] * 3 * n_pad;
  double re = 0, im = 0;
  for (int a = 0; a < lst.n; ++a) {
    const int atom = lst.idx ? lst.idx[a] : lst.first + a;
    double s, c;
    sincos(kx * P[atom] + ky * P[n_pad + atom] + kz * P[2 * n_pad + atom], &s, &c);
    re += c;
    im += s;
  }
  rho[(int64_t)f * n_k + k] = make_float2((float)re, (float)im);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static void check_frames(amdat_ctx* ctx, const int32_t* frames, int32_t n_frames) {
  AMDAT_REQUIRE(frames != nullptr && n_frames >= 1, "need >= 1 frame");
  AMDAT_REQUIRE(n_frames <= 65535, "at most 65535 frames per density");
  for (int i = 0; i < n_frames; ++i)
    AMDAT_REQUIRE(frames[i] >= 0 && frames[i] < ctx->n_frames, "frame index out of range");
}

static int4* fixed_turns(amdat_ctx* ctx, const Density& d, const ListEntry& e, float period,
                         DevBuf<int32_t>& d_frames) {
  d_frames.reserve(d.n_frames);
  AMDAT_CUDA(cudaMemcpyAsync(d_frames.ptr, d.frames.data(), d.n_frames * 4,
                             cudaMemcpyHostToDevice, ctx->stream));
  const int64_t n = (int64_t)d.n_frames * std::max(e.n, 1);
  int4* fx = (int4*)ctx->scratch2.reserve(n * sizeof(int4));
  if (e.n > 0) {
    const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->n_sm * 16);
    fixed_turns_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(
        ctx->w.ptr, ctx->n_pad, d.n_frames, d_frames.ptr, view(e), 1.0 / (double)period, fx);
    check_launch("fixed_turns_kernel");
    count_launch(ctx);
  }
  return fx;
}

// fixed-point phases of a list's atoms in the given (device) frames, into out
// [n_frames][n]; used by the adjoint kernels so they see the forward's phases
void fixed_turns_launch(amdat_ctx* ctx, const int32_t* d_frames, int32_t n_frames,
                        const ListEntry& e, float period, int4* out) {
  const int64_t n = (int64_t)n_frames * e.n;
  if (n == 0) return;
  const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->n_sm * 16);
  fixed_turns_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(ctx->w.ptr, ctx->n_pad, n_frames, d_frames,
                                                                view(e), 1.0 / (double)period, out);
  check_launch("fixed_turns_kernel");
  count_launch(ctx);
}

static int32_t store_density(amdat_ctx* ctx, Density* d) {
  const int32_t h = ctx->next_density++;
  ctx->densities[h] = d;
  return h;
}

Density& density(amdat_ctx* ctx, int32_t h) {
  auto it = ctx->densities.find(h);
  if (it == ctx->densities.end()) throw Error(AMDAT_ERR_ARGUMENT, "unknown density handle");
  return *it->second;
}

static void run_list_density(amdat_ctx* ctx, Density& d, float period, int32_t precision) {
  const ListEntry& e = list_entry(ctx, d.list);
  if (!d.rho) d.rho = rho_acquire(ctx, (size_t)d.n_frames * std::max(d.n_k, 1));
  DevBuf<int4> kv;
  kv.reserve(std::max(d.n_k, 1));
  std::vector<int4> hk(d.n_k);
  for (int k = 0; k < d.n_k; ++k)
    hk[k] = make_int4(d.kvec[3 * k], d.kvec[3 * k + 1], d.kvec[3 * k + 2], 0);
  if (d.n_k) AMDAT_CUDA(cudaMemcpyAsync(kv.ptr, hk.data(), d.n_k * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
  DevBuf<int32_t> d_frames;
  if (e.n == 0 || d.n_k == 0) {
    AMDAT_CUDA(cudaMemsetAsync(d.rho->ptr, 0, (size_t)d.n_frames * std::max(d.n_k, 1) * sizeof(float2), ctx->stream));
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    return;
  }
  if (precision == AMDAT_PLAIN_FP64) {
    ensure_fp64(ctx);
    d_frames.reserve(d.n_frames);
    AMDAT_CUDA(cudaMemcpyAsync(d_frames.ptr, d.frames.data(), d.n_frames * 4, cudaMemcpyHostToDevice, ctx->stream));
    dim3 grid((unsigned)ceil_div(d.n_k, 128), (unsigned)d.n_frames);
    KernelTimer kt(ctx, "rhok_plain_kernel");
    rhok_plain_kernel<<<grid, 128, 0, ctx->stream>>>(ctx->w64.ptr, ctx->n_pad, d_frames.ptr, view(e),
                                                      kv.ptr, d.n_k, 6.283185307179586476925286766559 / (double)period,
                                                      d.rho->ptr);
    check_launch("rhok_plain_kernel");
    count_launch(ctx);
  } else {
    int4* fx = fixed_turns(ctx, d, e, period, d_frames);
    dim3 grid((unsigned)ceil_div(d.n_k, RL_TILE), (unsigned)d.n_frames);
    KernelTimer kt(ctx, "rhok_list_kernel");
    rhok_list_kernel<<<grid, RL_THREADS, 0, ctx->stream>>>(fx, e.n, kv.ptr, d.n_k, d.rho->ptr);
    check_launch("rhok_list_kernel");
    count_launch(ctx);
  }
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
}

// half-space: nz > 0, or nz == 0 and (ny > 0, or ny == 0 and nx > 0)
static inline bool half_space(int nx, int ny, int nz) {
  return nz > 0 || (nz == 0 && (ny > 0 || (ny == 0 && nx > 0)));
}

struct LatticePlan {
  std::vector<int32_t> kvec;       // shell-sorted
  std::vector<int32_t> shell_off;
  std::vector<LatticeTile> tiles;
  std::vector<int32_t> entry_k;    // tile-major map to shell-sorted k, -1 = unused
};

// ---------------------------------------------------------------------------
// binned structure factor: Bin_Static_Analysis<Structure_Factor>
// (src/bin_static_analysis.h:69-111, src/control.cpp:2730-2737): bin b analyses
// the time-dependent list (list && bin b), i.e. at each frame the list members
// whose bin at that frame is b
// ---------------------------------------------------------------------------
constexpr int SKB_MAX_BINS = 4096;

// each frame's list members sorted by bin, list order kept within a bin: one
// warp per frame; seg[f][b] .. seg[f][b + 1] are bin b's slots of perm[f][]
// (positions in the list)
__global__ void __launch_bounds__(32)
    bins_segment_kernel(const int32_t* __restrict__ bin_map, int64_t n_pad, const int32_t* __restrict__ frames,
                        ListView lst, int32_t n_bins, int32_t* __restrict__ seg, int32_t* __restrict__ perm) {
  extern __shared__ int32_t cursor[];  // [n_bins]
  const int f = blockIdx.x, lane = threadIdx.x;
  const int32_t* B = bin_map + (int64_t)frames[f] * n_pad;
  for (int b = lane; b < n_bins; b += 32) cursor[b] = 0;
  __syncwarp();
  for (int i = lane; i < lst.n; i += 32) {
    const int b = B[lst.idx ? lst.idx[i] : lst.first + i];
    if (b >= 0 && b < n_bins) atomicAdd(&cursor[b], 1);
  }
  __syncwarp();
  int32_t* S = seg + (int64_t)f * (n_bins + 1);
  if (lane == 0) {
    int s = 0;
    for (int b = 0; b < n_bins; ++b) {
      const int c = cursor[b];
      cursor[b] = s;
      S[b] = s;
      s += c;
    }
    S[n_bins] = s;
  }
  __syncwarp();
  for (int i0 = 0; i0 < lst.n; i0 += 32) {
    const int i = i0 + lane;
    int b = -1;
    if (i < lst.n) {
      b = B[lst.idx ? lst.idx[i] : lst.first + i];
      if (b >= n_bins) b = -1;
    }
    // lanes of one bin take consecutive slots in lane (= list) order
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (b >= 0) perm[(int64_t)f * lst.n + cursor[b] + rank] = i;
    __syncwarp();
    if (b >= 0 && rank == 0) cursor[b] += __popc(peers);
    __syncwarp();
  }
}

// P[b][k] = sum over frames, in frame order, of |rho_b(f, k)|^2 in FP64, where
// rho_b(f, k) is the compensated FP32 sum of exp(i k.r) over bin b's members at
// frame f (the list-mode phases and accumulation)
__global__ void __launch_bounds__(RL_THREADS)
    sk_bins_kernel(const int4* __restrict__ fx, int32_t n_list, int32_t n_frames,
                   const int32_t* __restrict__ seg, const int32_t* __restrict__ perm, int32_t n_bins,
                   const int4* __restrict__ kv, int32_t n_k, double* __restrict__ P) {
  __shared__ int4 s_at[RL_ATOMS];
  const int b = blockIdx.y;
  const int k0 = blockIdx.x * RL_TILE;
  int4 n[RL_KPT];
  double p2[RL_KPT];
#pragma unroll
  for (int j = 0; j < RL_KPT; ++j) {
    const int k = k0 + j * RL_THREADS + threadIdx.x;
    n[j] = k < n_k ? kv[k] : make_int4(0, 0, 0, 0);
    p2[j] = 0.0;
  }
  for (int f = 0; f < n_frames; ++f) {
    const int s0 = seg[(int64_t)f * (n_bins + 1) + b], s1 = seg[(int64_t)f * (n_bins + 1) + b + 1];
    const int4* F = fx + (int64_t)f * n_list;
    const int32_t* Pm = perm + (int64_t)f * n_list;
    KC acc[RL_KPT];
    float pr[RL_KPT], pi[RL_KPT];
#pragma unroll
    for (int j = 0; j < RL_KPT; ++j) {
      acc[j] = KC{0.f, 0.f, 0.f, 0.f};
      pr[j] = pi[j] = 0.f;
    }
    int since_fold = 0;
    for (int a0 = s0; a0 < s1; a0 += RL_ATOMS) {
      const int na = min(RL_ATOMS, s1 - a0);
      __syncthreads();
      for (int i = threadIdx.x; i < na; i += RL_THREADS) s_at[i] = F[Pm[a0 + i]];
      __syncthreads();
      for (int a = 0; a < na; ++a) {
        const int4 q = s_at[a];
#pragma unroll
        for (int j = 0; j < RL_KPT; ++j) {
          const int32_t ph = (int32_t)((uint32_t)n[j].x * (uint32_t)q.x + (uint32_t)n[j].y * (uint32_t)q.y +
                                       (uint32_t)n[j].z * (uint32_t)q.z);
          float s, c;
          phase_sincos(ph, &s, &c);
          pr[j] += c;
          pi[j] += s;
        }
        if (++since_fold == 128) {
#pragma unroll
          for (int j = 0; j < RL_KPT; ++j) {
            kc_add(acc[j], pr[j], pi[j]);
            pr[j] = pi[j] = 0.f;
          }
          since_fold = 0;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < RL_KPT; ++j) {
      kc_add(acc[j], pr[j], pi[j]);
      const double re = (double)__fsub_rn(acc[j].sr, acc[j].cr), im = (double)__fsub_rn(acc[j].si, acc[j].ci);
      p2[j] += re * re + im * im;
    }
  }
#pragma unroll
  for (int j = 0; j < RL_KPT; ++j) {
    const int k = k0 + j * RL_THREADS + threadIdx.x;
    if (k < n_k) P[(int64_t)b * n_k + k] = p2[j];
  }
}

}  // namespace amdat
namespace amdat {
void rhok_tc_run(amdat_ctx* ctx, const TcPlan& P, const int4* fx, int32_t n_list, int32_t n_frames,
                 int32_t n_k, float2* rho);

struct LatticePlanDev {
  std::vector<int32_t> kvec, shell_off;
  DevBuf<LatticeTile> tiles;
  DevBuf<int32_t> entry_k;
  int32_t n_tiles = 0;
  TcPlan* tc = nullptr;  // tensor-core tiling, built at first use
  ~LatticePlanDev() { tc_plan_free(tc); }
};

void lattice_plans_free(amdat_ctx* ctx) {
  for (auto& kv : ctx->lattice_plans) delete kv.second;
  ctx->lattice_plans.clear();
}

TcPlan* lattice_tc_plan(amdat_ctx* ctx, const std::string& lattice_key) {
  auto it = ctx->lattice_plans.find(lattice_key);
  AMDAT_REQUIRE(it != ctx->lattice_plans.end(), "lattice plan not found");
  if (!it->second->tc) it->second->tc = tc_plan_build(it->second->kvec);
  return it->second->tc;
}

// tcgen05 kernel on compute capability 10.x unless AMDAT_RHOK_KERNEL=fp32
static bool use_tensor_cores(amdat_ctx* ctx) {
  const char* e = std::getenv("AMDAT_RHOK_KERNEL");
  if (e && std::strcmp(e, "fp32") == 0) return false;
  int major = 0;
  AMDAT_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx->device));
  return major == 10;
}

bool tc_enabled(amdat_ctx* ctx) { return use_tensor_cores(ctx); }

static LatticePlan plan_lattice(float kmax, float dk, float period) {
  const double two_pi = 6.283185307179586476925286766559;
  const double R = (double)kmax * (double)period / two_pi;  // |n| <= R
  AMDAT_REQUIRE(R >= 1.0 && R < 1024.0, "kmax*period/(2 pi) must be in [1, 1024)");
  const int nmax = (int)std::floor(R);
  const double R2 = R * R;
  const int n_shells = (int)std::floor((double)kmax / (double)dk) + 1;
  AMDAT_REQUIRE(n_shells >= 1 && n_shells <= (1 << 20), "bad shell width");
  LatticePlan P;
  // collect vectors tile by tile, then sort by shell (stable: tile order within shell)
  struct V {
    int32_t shell, nx, ny, nz;
    int64_t entry;
  };
  std::vector<V> vs;
  for (int x0 = -nmax; x0 <= nmax; x0 += LT_NX)
    for (int y0 = -nmax; y0 <= nmax; y0 += LT_NY) {
      int nzm = -1;
      for (int nx = x0; nx < x0 + LT_NX; ++nx)
        for (int ny = y0; ny < y0 + LT_NY; ++ny) {
          const double r2 = R2 - (double)nx * nx - (double)ny * ny;
          if (r2 >= 0) nzm = std::max(nzm, (int)std::floor(std::sqrt(r2)));
        }
      for (int z0 = 0; z0 <= nzm; z0 += LT_NZ) {
        const int32_t entry0 = (int32_t)P.entry_k.size();
        P.tiles.push_back(LatticeTile{x0, y0, z0, entry0});
        P.entry_k.resize(P.entry_k.size() + LT_ROWS * LT_NZ, -1);
        for (int r = 0; r < LT_ROWS; ++r)
          for (int c = 0; c < LT_NZ; ++c) {
            const int nx = x0 + r % LT_NX, ny = y0 + r / LT_NX, nz = z0 + c;
            if (std::abs(nx) > nmax || std::abs(ny) > nmax || nz > nmax) continue;
            const double n2 = (double)nx * nx + (double)ny * ny + (double)nz * nz;
            if (n2 > R2 || !half_space(nx, ny, nz)) continue;
            const double kk = two_pi * std::sqrt(n2) / (double)period;
            const int s = std::min(n_shells - 1, (int)std::floor(kk / (double)dk));
            vs.push_back(V{s, nx, ny, nz, (int64_t)entry0 + r * LT_NZ + c});
          }
      }
    }
  std::stable_sort(vs.begin(), vs.end(), [](const V& a, const V& b) { return a.shell < b.shell; });
  AMDAT_REQUIRE(vs.size() < (size_t)INT32_MAX / 3, "too many lattice vectors");
  P.kvec.resize(vs.size() * 3);
  P.shell_off.assign(n_shells + 1, 0);
  for (size_t k = 0; k < vs.size(); ++k) {
    P.kvec[3 * k] = vs[k].nx;
    P.kvec[3 * k + 1] = vs[k].ny;
    P.kvec[3 * k + 2] = vs[k].nz;
    P.entry_k[vs[k].entry] = (int32_t)k;
    P.shell_off[vs[k].shell + 1]++;
  }
  for (int s = 0; s < n_shells; ++s) P.shell_off[s + 1] += P.shell_off[s];
  return P;
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_wave_density(amdat_ctx* ctx, int32_t list, const int32_t* kvec_n, int32_t n_k,
                                float period, const int32_t* frames, int32_t n_frames,
                                int32_t precision, int32_t* handle) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(handle != nullptr, "null handle pointer");
    AMDAT_REQUIRE(n_k >= 0 && (n_k == 0 || kvec_n != nullptr), "bad vector list");
    AMDAT_REQUIRE(period > 0.0f, "period must be positive");
    AMDAT_REQUIRE(precision == AMDAT_MIXED || precision == AMDAT_PLAIN_FP64, "bad precision");
    check_frames(ctx, frames, n_frames);
    list_entry(ctx, list);
    for (int i = 0; i < 3 * n_k; ++i) AMDAT_REQUIRE(std::abs(kvec_n[i]) < (1 << 20), "lattice index too large");
    auto* d = new Density();
    d->list = list;
    d->n_k = n_k;
    d->n_frames = n_frames;
    d->period = period;
    d->n_list = list_entry(ctx, list).n;
    d->frames.assign(frames, frames + n_frames);
    d->kvec.assign(kvec_n, kvec_n + 3 * (size_t)n_k);
    try {
      run_list_density(ctx, *d, period, precision);
    } catch (...) {
      rho_release(ctx, d->rho);
      delete d;
      throw;
    }
    *handle = store_density(ctx, d);
  });
}

amdat_status amdat_wave_density_lattice(amdat_ctx* ctx, int32_t list, float kmax, float dk,
                                        float period, const int32_t* frames, int32_t n_frames,
                                        int32_t precision, int32_t* handle, int32_t* n_k,
                                        int32_t* n_shells) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(handle != nullptr, "null handle pointer");
    AMDAT_REQUIRE(kmax > 0.0f && dk > 0.0f && period > 0.0f, "kmax, dk, period must be positive");
    AMDAT_REQUIRE(precision == AMDAT_MIXED || precision == AMDAT_PLAIN_FP64, "bad precision");
    check_frames(ctx, frames, n_frames);
    const ListEntry& e = list_entry(ctx, list);
    // plans depend only on (kmax, dk, period): build once, keep on the device
    char key[96];
    std::snprintf(key, sizeof(key), "%a/%a/%a", (double)kmax, (double)dk, (double)period);
    auto it = ctx->lattice_plans.find(key);
    if (it == ctx->lattice_plans.end()) {
      LatticePlan P = plan_lattice(kmax, dk, period);
      auto* pd = new LatticePlanDev();
      pd->kvec = std::move(P.kvec);
      pd->shell_off = std::move(P.shell_off);
      pd->n_tiles = (int32_t)P.tiles.size();
      pd->tiles.reserve(P.tiles.size());
      pd->entry_k.reserve(P.entry_k.size());
      AMDAT_CUDA(cudaMemcpy(pd->tiles.ptr, P.tiles.data(), P.tiles.size() * sizeof(LatticeTile), cudaMemcpyHostToDevice));
      AMDAT_CUDA(cudaMemcpy(pd->entry_k.ptr, P.entry_k.data(), P.entry_k.size() * 4, cudaMemcpyHostToDevice));
      it = ctx->lattice_plans.emplace(key, pd).first;
    }
    const LatticePlanDev& P = *it->second;
    auto* d = new Density();
    d->list = list;
    d->n_k = (int32_t)(P.kvec.size() / 3);
    d->n_frames = n_frames;
    d->n_shells = (int32_t)P.shell_off.size() - 1;
    d->period = period;
    d->lattice_key = key;
    d->n_list = e.n;
    d->frames.assign(frames, frames + n_frames);
    d->kvec = P.kvec;
    d->shell_off = P.shell_off;
    try {
      if (precision == AMDAT_PLAIN_FP64 || e.n == 0) {
        run_list_density(ctx, *d, period, precision);
      } else {
        d->rho = rho_acquire(ctx, (size_t)n_frames * std::max(d->n_k, 1));
        DevBuf<int32_t> d_frames;
        int4* fx = fixed_turns(ctx, *d, e, period, d_frames);
        if (use_tensor_cores(ctx)) {
          LatticePlanDev& pw = *it->second;
          if (!pw.tc) pw.tc = tc_plan_build(pw.kvec);
          rhok_tc_run(ctx, *pw.tc, fx, e.n, n_frames, d->n_k, d->rho->ptr);
        } else {
          dim3 grid((unsigned)P.n_tiles, (unsigned)n_frames);
          KernelTimer kt(ctx, "rhok_lattice_kernel");
          rhok_lattice_kernel<<<grid, LT_THREADS, 0, ctx->stream>>>(fx, e.n, P.tiles.ptr, P.entry_k.ptr,
                                                                   d->n_k, d->rho->ptr);
          check_launch("rhok_lattice_kernel");
          count_launch(ctx);
        }
        AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
      }
    } catch (...) {
      rho_release(ctx, d->rho);
      delete d;
      throw;
    }
    *handle = store_density(ctx, d);
    if (n_k) *n_k = d->n_k;
    if (n_shells) *n_shells = d->n_shells;
  });
}

amdat_status amdat_wave_density_vectors(amdat_ctx* ctx, int32_t handle, int32_t* kvec_n,
                                        int32_t* shell_offsets) {
  return guarded([&] {
    check_ctx(ctx);
    Density& d = density(ctx, handle);
    if (kvec_n) std::memcpy(kvec_n, d.kvec.data(), d.kvec.size() * 4);
    if (shell_offsets && !d.shell_off.empty())
      std::memcpy(shell_offsets, d.shell_off.data(), d.shell_off.size() * 4);
  });
}

amdat_status amdat_wave_density_read(amdat_ctx* ctx, int32_t handle, int32_t out_flags,
                                     float* rho) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(rho != nullptr, "null output");
    Density& d = density(ctx, handle);
    AMDAT_CUDA(cudaMemcpyAsync(rho, d.rho->ptr, (size_t)d.n_frames * d.n_k * sizeof(float2),
                               out_flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice
                                                             : cudaMemcpyDeviceToHost,
                               ctx->stream));
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

amdat_status amdat_wave_density_free(amdat_ctx* ctx, int32_t handle) {
  return guarded([&] {
    check_ctx(ctx);
    auto it = ctx->densities.find(handle);
    if (it == ctx->densities.end()) throw Error(AMDAT_ERR_ARGUMENT, "unknown density handle");
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    rho_release(ctx, it->second->rho);
    delete it->second;
    ctx->densities.erase(it);
  });
}

amdat_status amdat_structure_factor_bins(amdat_ctx* ctx, int32_t list, int32_t bins,
                                         const int32_t* kvec_n, int32_t n_k, const int32_t* shell_offsets,
                                         int32_t n_shells, float period, const int32_t* frames,
                                         int32_t n_frames, double* s_sum, int64_t* n_atoms) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(s_sum != nullptr && n_atoms != nullptr, "null output");
    AMDAT_REQUIRE(n_k >= 0 && (n_k == 0 || kvec_n != nullptr), "bad vector list");
    AMDAT_REQUIRE(shell_offsets != nullptr && n_shells >= 1, "bad shell offsets");
    AMDAT_REQUIRE(shell_offsets[0] == 0 && shell_offsets[n_shells] == n_k, "shell offsets must span 0..n_k");
    for (int s = 0; s < n_shells; ++s)
      AMDAT_REQUIRE(shell_offsets[s + 1] >= shell_offsets[s], "shell offsets must not decrease");
    AMDAT_REQUIRE(period > 0.0f, "period must be positive");
    check_frames(ctx, frames, n_frames);
    for (int i = 0; i < 3 * n_k; ++i) AMDAT_REQUIRE(std::abs(kvec_n[i]) < (1 << 20), "lattice index too large");
    const ListEntry& e = list_entry(ctx, list);
    auto it = ctx->bin_maps.find(bins);
    AMDAT_REQUIRE(it != ctx->bin_maps.end(), "unknown bin map handle");
    const BinMap& m = *it->second;
    AMDAT_REQUIRE(m.n_frames == ctx->n_frames && m.n_pad == ctx->n_pad, "bin map made for another trajectory");
    const int32_t B = m.nx * m.ny * m.nz;
    AMDAT_REQUIRE(B >= 1 && B <= SKB_MAX_BINS, "at most 4096 bins");
    std::vector<int32_t> fr(frames, frames + n_frames);
    std::vector<int4> kv4((size_t)std::max(n_k, 1));
    for (int k = 0; k < n_k; ++k) kv4[k] = make_int4(kvec_n[3 * k], kvec_n[3 * k + 1], kvec_n[3 * k + 2], 0);
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const int64_t nl = std::max(e.n, 1);
    size_t o = 0;
    const size_t o_fr = o; o = align(o + (size_t)std::max(n_frames, 1) * 4);
    const size_t o_kv = o; o = align(o + kv4.size() * sizeof(int4));
    const size_t o_seg = o; o = align(o + (size_t)std::max(n_frames, 1) * (B + 1) * 4);
    const size_t o_perm = o; o = align(o + (size_t)std::max(n_frames, 1) * nl * 4);
    const size_t o_p = o; o = align(o + (size_t)B * std::max(n_k, 1) * 8);
    unsigned char* base = ctx->scratch.reserve(o);
    int4* fx = (int4*)ctx->scratch2.reserve((size_t)std::max(n_frames, 1) * nl * sizeof(int4));
    if (n_frames > 0)
      AMDAT_CUDA(cudaMemcpyAsync(base + o_fr, fr.data(), (size_t)n_frames * 4, cudaMemcpyHostToDevice, ctx->stream));
    AMDAT_CUDA(cudaMemcpyAsync(base + o_kv, kv4.data(), kv4.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
    std::vector<double> P((size_t)B * std::max(n_k, 1), 0.0);
    std::vector<int32_t> seg((size_t)std::max(n_frames, 1) * (B + 1), 0);
    if (n_frames > 0 && e.n > 0) {
      fixed_turns_launch(ctx, (const int32_t*)(base + o_fr), n_frames, e, period, fx);
      bins_segment_kernel<<<(unsigned)n_frames, 32, (size_t)B * 4, ctx->stream>>>(
          m.bin.ptr, m.n_pad, (const int32_t*)(base + o_fr), view(e), B, (int32_t*)(base + o_seg),
          (int32_t*)(base + o_perm));
      check_launch("bins_segment_kernel");
      count_launch(ctx);
      if (n_k > 0) {
        AMDAT_REQUIRE(B <= 65535, "too many bins for one launch");
        dim3 grid((unsigned)ceil_div(n_k, RL_TILE), (unsigned)B);
        KernelTimer kt(ctx, "sk_bins_kernel");
        sk_bins_kernel<<<grid, RL_THREADS, 0, ctx->stream>>>(fx, e.n, n_frames, (const int32_t*)(base + o_seg),
                                                            (const int32_t*)(base + o_perm), B,
                                                            (const int4*)(base + o_kv), n_k, (double*)(base + o_p));
        check_launch("sk_bins_kernel");
        count_launch(ctx);
        AMDAT_CUDA(cudaMemcpyAsync(P.data(), base + o_p, (size_t)B * n_k * 8, cudaMemcpyDeviceToHost, ctx->stream));
      }
      AMDAT_CUDA(cudaMemcpyAsync(seg.data(), base + o_seg, (size_t)n_frames * (B + 1) * 4, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    }
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    // shell means in a fixed order (FP64), member counts summed over frames
    for (int b = 0; b < B; ++b) {
      for (int s = 0; s < n_shells; ++s) {
        const int h = shell_offsets[s + 1] - shell_offsets[s];
        double acc = 0.0;
        for (int k = shell_offsets[s]; k < shell_offsets[s + 1]; ++k) acc += P[(size_t)b * n_k + k];
        s_sum[(size_t)b * n_shells + s] = h ? acc / h : 0.0;
      }
      int64_t na = 0;
      for (int f = 0; f < n_frames; ++f) na += seg[(size_t)f * (B + 1) + b + 1] - seg[(size_t)f * (B + 1) + b];
      n_atoms[b] = na;
    }
  });
}

}  // extern "C"
