// Differentiable structure: a Gaussian-smoothed pair histogram and the
// adjoints (gradients with respect to positions) of it and of the static
// structure factor.  The reference has only the hard-binned forward parts
// (Radial_Distribution_Function::listkernel, src/radial_distribution_function.cpp:233-285;
// Structure_Factor::listkernel, src/structure_factor.cpp:293-320); the
// smoothing kernel and both adjoints are this engine's own.
//
// Smoothed pair histogram of one list, bin centres r_b = (b + 1/2) r_max / n_bins:
//     h_b = sum_t sum_{i<j} G(r_b - r_ij),  G(x) = exp(-x^2 / 2 sigma^2) / (sqrt(2 pi) sigma)
// with r_ij the minimum-image distance (FP32, d - L rint(d / L)) and pairs
// beyond r_max + 6 sigma skipped; each term is rounded to a fixed-point integer
// (relative step below 1e-9 of the largest term) and summed exactly.  Adjoint for w_b = dLoss/dh_b:
//     psi(r) = sum_b w_b (r_b - r) / sigma^2 G(r_b - r)
//     dLoss/dr_i(t) = sum_{j != i} psi(r_ij) (r_i - r_j) / r_ij
// with the pair loop recomputed (nothing is stored between the passes).  A
// thread owns one atom and visits every other atom, so every gradient element
// has a single writer: no atomics, deterministic.
//
// Structure-factor adjoint.  With S_raw_s = sum_t sum_{k in s} |rho_k(t)|^2 / H_s
// and w_s = dLoss/dS_raw_s, write c_k = (2 w_s / H_s) conj(rho_k(t)); then
//     dLoss/dr_j(t) = -(2 pi / L) Im sum_k n_k c_k exp(i 2 pi n_k . r_j / L).
// Two kernels evaluate that sum:
//   sk_adjoint_columns_kernel  vectors grouped into lattice columns (fixed nx, ny,
//                              consecutive nz): exp(i k.r) is advanced along nz by
//                              one complex multiplication per vector, re-anchored
//                              from the exact fixed-point phase every 64 steps.
//                              Used when the columns average >= 8 vectors (the
//                              |k| <= kmax lattice densities).
//   sk_adjoint_direct_kernel   one sincospif per (atom, vector) for arbitrary
//                              lists (e.g. thin q-vector shells).
// Both use the forward's fixed-point phases and fold per-tile sums into
// Kahan-compensated FP32 accumulators.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "engine.h"
#include "tc_tiles.h"

namespace amdat {

void sk_adjoint_tc_run(amdat_ctx* ctx, const TcPlan& P, const int4* fx, int32_t n, int32_t F,
                       const float2* rho, int32_t n_k, const float* d_u, float max_u, float period,
                       float* grad);

struct SGList {
  int32_t n;
  int32_t first;
  const int32_t* idx;
};

static SGList sglist(const ListEntry& e) { return SGList{e.n, e.first, e.contiguous ? nullptr : e.idx.ptr}; }

__device__ __forceinline__ int sg_member(const SGList& l, int a) { return l.idx ? l.idx[a] : l.first + a; }

__device__ __forceinline__ float min_image(float d, float L, float inv_l) {
  return fmaf(-L, rintf(d * inv_l), d);
}

constexpr int SG_THREADS = 256;
constexpr int SG_JT = 1024;
constexpr float SG_CUT = 6.0f;  // kernel support in units of sigma
constexpr float INV_SQRT_2PI = 0.3989422804014327f;

struct SGParams {
  const float* w;  // wrapped planes [T][3][n_pad]
  int64_t n_pad;
  SGList lst;
  const int32_t* frames;
  float3 box, inv_box;
  float sigma, bin, cut2;
  int32_t n_bins, span;
  double* h;          // forward output [n_bins] (accumulated)
  const double* wgt;  // adjoint input [n_bins]
  float* grad;        // adjoint output [n_frames][n][3]
};

__device__ __forceinline__ void stage_atoms(const SGParams& p, const float* P, int j0, int nj, float* sx,
                                            float* sy, float* sz) {
  for (int t = threadIdx.x; t < nj; t += blockDim.x) {
    const int a = sg_member(p.lst, j0 + t);
    sx[t] = P[a];
    sy[t] = P[p.n_pad + a];
    sz[t] = P[2 * p.n_pad + a];
  }
}

// Gaussian terms of one pair over its bins b0..b1, x_b = (b + 1/2) bin - r:
// G_b = exp(-x_b^2 / 2 sigma^2) by the exact recurrence G_{b+1} = G_b R_b,
// R_{b+1} = R_b Q (two exponentials per pair instead of one per bin) when
// the bin is at most 2 sigma wide (the factors then stay within FP32 range),
// else one exponential per bin.  f(b, x, G) receives each term.
template <class F>
__device__ __forceinline__ void gauss_bins(const SGParams& p, float r, float inv2s2, bool recur, F f) {
  const int bc = (int)(r * (1.0f / p.bin));
  const int b0 = max(0, bc - p.span), b1 = min(p.n_bins - 1, bc + p.span);
  if (b0 > b1) return;
  float x = fmaf((float)b0 + 0.5f, p.bin, -r);
  if (recur) {
    float G = __expf(-x * x * inv2s2);
    float R = __expf(-(2.0f * x * p.bin + p.bin * p.bin) * inv2s2);
    const float Q = __expf(-2.0f * p.bin * p.bin * inv2s2);
    for (int b = b0; b <= b1; ++b) {
      f(b, x, G);
      G *= R;
      R *= Q;
      x += p.bin;
    }
  } else {
    for (int b = b0; b <= b1; ++b) {
      f(b, x, __expf(-x * x * inv2s2));
      x += p.bin;
    }
  }
}

constexpr int SG_WARPS = SG_THREADS / 32;
constexpr int SG_Q = 64;  // per-warp queue of in-range pairs

// forward: unordered pairs j > i.  In-range pairs (about 2 % of all pairs at
// the usual cutoffs) are compacted into a per-warp queue with ballots and
// their bins are processed 32 at a time, so the bin loop runs with every lane
// busy.  Each Gaussian term is rounded once to a fixed-point integer (scale
// 2^q chosen by the host so that a block's sum cannot overflow 63 bits) and
// added with 64-bit shared-memory integer atomics: the block histogram is
// exact and independent of the order of the additions, so the forward is
// deterministic and finite differences of it see only the terms that change.
__global__ void __launch_bounds__(SG_THREADS) gsmooth_kernel(SGParams p, float qscale) {
  extern __shared__ double sh_d[];  // [n_bins] as unsigned 64-bit fixed point
  unsigned long long* sh_q = reinterpret_cast<unsigned long long*>(sh_d);
  __shared__ float sx[SG_JT], sy[SG_JT], sz[SG_JT];
  __shared__ float q_r[SG_WARPS][SG_Q];
  const int f = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* P = p.w + (int64_t)p.frames[f] * 3 * p.n_pad;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x) sh_q[b] = 0ull;
  const int i0 = blockIdx.x * SG_THREADS, i = i0 + threadIdx.x;
  const bool live = i < p.lst.n;
  float xi = 0.f, yi = 0.f, zi = 0.f;
  if (live) {
    const int a = sg_member(p.lst, i);
    xi = P[a];
    yi = P[p.n_pad + a];
    zi = P[2 * p.n_pad + a];
  }
  const float inv2s2 = 0.5f / (p.sigma * p.sigma);
  const float qnorm = qscale * INV_SQRT_2PI / p.sigma;
  const bool recur = p.bin <= 2.0f * p.sigma;
  const unsigned below = (1u << lane) - 1u;
  auto flush = [&](int count) {  // lanes < count take one queued pair each
    if (lane < count)
      gauss_bins(p, q_r[warp][lane], inv2s2, recur, [&](int b, float, float G) {
        atomicAdd(sh_q + b, (unsigned long long)__float2ll_rn(qnorm * G));
      });
  };
  int qn = 0;  // warp-uniform queue length
  for (int j0 = i0; j0 < p.lst.n; j0 += SG_JT) {
    const int nj = min(SG_JT, p.lst.n - j0);
    __syncthreads();
    stage_atoms(p, P, j0, nj, sx, sy, sz);
    __syncthreads();
    for (int t = 0; t < nj; ++t) {
      const float dx = min_image(sx[t] - xi, p.box.x, p.inv_box.x);
      const float dy = min_image(sy[t] - yi, p.box.y, p.inv_box.y);
      const float dz = min_image(sz[t] - zi, p.box.z, p.inv_box.z);
      const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      const bool in = live && j0 + t > i && r2 < p.cut2;
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) q_r[warp][qn + __popc(m & below)] = sqrtf(r2);
      qn += __popc(m);
      if (qn >= 32) {
        __syncwarp();
        flush(32);
        __syncwarp();
        if (lane < qn - 32) q_r[warp][lane] = q_r[warp][32 + lane];
        __syncwarp();
        qn -= 32;
      }
    }
  }
  __syncwarp();
  flush(qn);
  __syncthreads();
  const double inv_q = 1.0 / (double)qscale;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x)
    if (sh_q[b]) atomicAdd(p.h + b, (double)sh_q[b] * inv_q);
}

// adjoint: each atom i gathers psi(r_ij) (r_i - r_j) / r_ij over every j != i.
// In-range pairs are compacted into a per-warp queue (the pair's minimum-image
// vector, r and its owner lane); the warp evaluates psi for 32 queued pairs
// at a time, then every owner adds its own entries in queue order, so every
// gradient element still has a single writer and a fixed summation order.
__global__ void __launch_bounds__(SG_THREADS) gsmooth_adjoint_kernel(SGParams p) {
  extern __shared__ double sh_d[];  // [n_bins] weights as FP32
  float* sh_w = (float*)sh_d;
  __shared__ float sx[SG_JT], sy[SG_JT], sz[SG_JT];
  __shared__ float4 q_v[SG_WARPS][SG_Q];  // (dx, dy, dz, r); after a flush: (s dx, s dy, s dz, -)
  __shared__ unsigned char q_o[SG_WARPS][SG_Q];
  const int f = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* P = p.w + (int64_t)p.frames[f] * 3 * p.n_pad;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x) sh_w[b] = (float)p.wgt[b];
  const int i = blockIdx.x * SG_THREADS + threadIdx.x;
  const bool live = i < p.lst.n;
  float xi = 0.f, yi = 0.f, zi = 0.f;
  if (live) {
    const int a = sg_member(p.lst, i);
    xi = P[a];
    yi = P[p.n_pad + a];
    zi = P[2 * p.n_pad + a];
  }
  const float inv_s2 = 1.0f / (p.sigma * p.sigma);
  const float inv2s2 = 0.5f * inv_s2;
  const float scale = INV_SQRT_2PI / p.sigma * inv_s2;
  const bool recur = p.bin <= 2.0f * p.sigma;
  const unsigned below = (1u << lane) - 1u;
  float g[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
  auto flush = [&](int count) {
    if (lane < count) {
      float4 v = q_v[warp][lane];
      float psi = 0.f;
      gauss_bins(p, v.w, inv2s2, recur, [&](int b, float x, float G) { psi = fmaf(sh_w[b] * x, G, psi); });
      const float s = psi * scale / v.w;
      q_v[warp][lane] = make_float4(s * v.x, s * v.y, s * v.z, 0.f);
    }
    __syncwarp();
    // owners add their entries in queue order (compensated)
    float part[3] = {0.f, 0.f, 0.f};
    for (int e = 0; e < count; ++e)
      if (q_o[warp][e] == lane) {
        const float4 v = q_v[warp][e];
        part[0] += v.x;
        part[1] += v.y;
        part[2] += v.z;
      }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float y = __fsub_rn(part[d], c[d]), t = __fadd_rn(g[d], y);
      c[d] = __fsub_rn(__fsub_rn(t, g[d]), y);
      g[d] = t;
    }
  };
  int qn = 0;
  __syncthreads();
  for (int j0 = 0; j0 < p.lst.n; j0 += SG_JT) {
    const int nj = min(SG_JT, p.lst.n - j0);
    __syncthreads();
    stage_atoms(p, P, j0, nj, sx, sy, sz);
    __syncthreads();
    for (int t = 0; t < nj; ++t) {
      // d = r_i - r_j (minimum image)
      const float dx = min_image(xi - sx[t], p.box.x, p.inv_box.x);
      const float dy = min_image(yi - sy[t], p.box.y, p.inv_box.y);
      const float dz = min_image(zi - sz[t], p.box.z, p.inv_box.z);
      const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      const bool in = live && j0 + t != i && r2 < p.cut2 && r2 > 0.f;
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int pos = qn + __popc(m & below);
        q_v[warp][pos] = make_float4(dx, dy, dz, sqrtf(r2));
        q_o[warp][pos] = (unsigned char)lane;
      }
      qn += __popc(m);
      if (qn >= 32) {
        __syncwarp();
        flush(32);
        __syncwarp();
        if (lane < qn - 32) {
          q_v[warp][lane] = q_v[warp][32 + lane];
          q_o[warp][lane] = q_o[warp][32 + lane];
        }
        __syncwarp();
        qn -= 32;
      }
    }
  }
  __syncwarp();
  flush(qn);
  if (live) {
    float* out = p.grad + ((int64_t)f * p.lst.n + i) * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) out[d] = __fsub_rn(g[d], c[d]);
  }
}

// ---------------------------------------------------------------------------
// cell lists: boxes at least three cutoffs wide on every axis are cut into
// cells no smaller than the cutoff; an atom's partners within the cutoff lie
// in its own or the 26 neighbouring cells (periodic).  Per frame the list's
// atoms are counted into cells, scattered, and each cell's atoms are put in
// ascending list order, so every loop below runs in a fixed order.
// ---------------------------------------------------------------------------
struct SGCells {
  int3 nc;
  float3 lo, inv_cell;
  const int32_t* start;  // [n_cells + 1]
  const int32_t* order;  // sorted slot -> list index
  const float4* pos;     // sorted slot -> wrapped position
};

__device__ __forceinline__ int cell_axis(float x, float lo, float inv_cell, int n) {
  const int c = (int)((x - lo) * inv_cell);
  return min(max(c, 0), n - 1);
}

__global__ void cell_assign_kernel(const float* __restrict__ P, int64_t n_pad, SGList lst, float3 lo,
                                   float3 inv_cell, int3 nc, int32_t* __restrict__ cell_of,
                                   int32_t* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= lst.n) return;
  const int a = sg_member(lst, i);
  const int cx = cell_axis(P[a], lo.x, inv_cell.x, nc.x);
  const int cy = cell_axis(P[n_pad + a], lo.y, inv_cell.y, nc.y);
  const int cz = cell_axis(P[2 * n_pad + a], lo.z, inv_cell.z, nc.z);
  const int c = (cz * nc.y + cy) * nc.x + cx;
  cell_of[i] = c;
  atomicAdd(count + c, 1);
}

// exclusive scan of count[0..n) into start[0..n] (one block)
__global__ void cell_scan_kernel(const int32_t* __restrict__ count, int32_t n, int32_t* __restrict__ start,
                                 int32_t* __restrict__ cursor) {
  __shared__ int32_t s_part[1024];
  __shared__ int32_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    s_part[threadIdx.x] = i < n ? count[i] : 0;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int v = threadIdx.x >= off ? s_part[threadIdx.x - off] : 0;
      __syncthreads();
      s_part[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < n) {
      const int excl = s_carry + s_part[threadIdx.x] - count[i];
      start[i] = excl;
      cursor[i] = excl;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_carry += s_part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) start[n] = s_carry;
}

__global__ void cell_scatter_kernel(const int32_t* __restrict__ cell_of, int32_t n, int32_t* __restrict__ cursor,
                                    int32_t* __restrict__ order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) order[atomicAdd(cursor + cell_of[i], 1)] = i;
}

// ascending list order inside each cell, then the sorted positions
__global__ void cell_sort_kernel(const int32_t* __restrict__ start, int32_t n_cells, int32_t* __restrict__ order,
                                 const float* __restrict__ P, int64_t n_pad, SGList lst, float4* __restrict__ pos) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  const int b = start[c], e = start[c + 1];
  for (int k = b + 1; k < e; ++k) {
    const int v = order[k];
    int m = k - 1;
    while (m >= b && order[m] > v) {
      order[m + 1] = order[m];
      --m;
    }
    order[m + 1] = v;
  }
  for (int k = b; k < e; ++k) {
    const int a = sg_member(lst, order[k]);
    pos[k] = make_float4(P[a], P[n_pad + a], P[2 * n_pad + a], 0.f);
  }
}

// neighbour cell `off` (0..26) of the cell holding p, periodic
__device__ __forceinline__ int neighbour_cell(const SGCells& C, float4 p, int off) {
  const int dx = off % 3 - 1, dy = (off / 3) % 3 - 1, dz = off / 9 - 1;
  int cx = cell_axis(p.x, C.lo.x, C.inv_cell.x, C.nc.x) + dx;
  int cy = cell_axis(p.y, C.lo.y, C.inv_cell.y, C.nc.y) + dy;
  int cz = cell_axis(p.z, C.lo.z, C.inv_cell.z, C.nc.z) + dz;
  cx += cx < 0 ? C.nc.x : (cx >= C.nc.x ? -C.nc.x : 0);
  cy += cy < 0 ? C.nc.y : (cy >= C.nc.y ? -C.nc.y : 0);
  cz += cz < 0 ? C.nc.z : (cz >= C.nc.z ? -C.nc.z : 0);
  return (cz * C.nc.y + cy) * C.nc.x + cx;
}

// forward over cells: thread per sorted slot, partners j > i (list order) in
// the 27 cells; queue and bins as in gsmooth_kernel
__global__ void __launch_bounds__(SG_THREADS) gsmooth_cells_kernel(SGParams p, SGCells C, float qscale) {
  extern __shared__ double sh_d[];
  unsigned long long* sh_q = reinterpret_cast<unsigned long long*>(sh_d);
  __shared__ float q_r[SG_WARPS][SG_Q];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x) sh_q[b] = 0ull;
  __syncthreads();
  const int slot = blockIdx.x * SG_THREADS + threadIdx.x;
  const bool live = slot < p.lst.n;
  const int i = live ? C.order[slot] : -1;
  const float4 pi = live ? C.pos[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float inv2s2 = 0.5f / (p.sigma * p.sigma);
  const float qnorm = qscale * INV_SQRT_2PI / p.sigma;
  const bool recur = p.bin <= 2.0f * p.sigma;
  const unsigned below = (1u << lane) - 1u;
  auto flush = [&](int count) {
    if (lane < count)
      gauss_bins(p, q_r[warp][lane], inv2s2, recur, [&](int b, float, float G) {
        atomicAdd(sh_q + b, (unsigned long long)__float2ll_rn(qnorm * G));
      });
  };
  int qn = 0;
  for (int off = 0; off < 27; ++off) {
    const int nb = live ? neighbour_cell(C, pi, off) : 0;
    const int cs = live ? C.start[nb] : 0, len = live ? C.start[nb + 1] - cs : 0;
    const int maxlen = __reduce_max_sync(0xffffffffu, len);
    for (int k = 0; k < maxlen; ++k) {
      bool in = false;
      float r2 = 0.f;
      if (k < len) {
        const int j = C.order[cs + k];
        const float4 pj = C.pos[cs + k];
        const float dx = min_image(pj.x - pi.x, p.box.x, p.inv_box.x);
        const float dy = min_image(pj.y - pi.y, p.box.y, p.inv_box.y);
        const float dz = min_image(pj.z - pi.z, p.box.z, p.inv_box.z);
        r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        in = j > i && r2 < p.cut2;
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) q_r[warp][qn + __popc(m & below)] = sqrtf(r2);
      qn += __popc(m);
      if (qn >= 32) {
        __syncwarp();
        flush(32);
        __syncwarp();
        if (lane < qn - 32) q_r[warp][lane] = q_r[warp][32 + lane];
        __syncwarp();
        qn -= 32;
      }
    }
  }
  __syncwarp();
  flush(qn);
  __syncthreads();
  const double inv_q = 1.0 / (double)qscale;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x)
    if (sh_q[b]) atomicAdd(p.h + b, (double)sh_q[b] * inv_q);
}

// adjoint over cells: thread per sorted slot, every partner j != i in the 27
// cells, owner-ordered sums as in gsmooth_adjoint_kernel
__global__ void __launch_bounds__(SG_THREADS) gsmooth_cells_adjoint_kernel(SGParams p, SGCells C, int32_t frame) {
  extern __shared__ double sh_d[];
  float* sh_w = (float*)sh_d;
  __shared__ float4 q_v[SG_WARPS][SG_Q];
  __shared__ unsigned char q_o[SG_WARPS][SG_Q];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x) sh_w[b] = (float)p.wgt[b];
  __syncthreads();
  const int slot = blockIdx.x * SG_THREADS + threadIdx.x;
  const bool live = slot < p.lst.n;
  const int i = live ? C.order[slot] : -1;
  const float4 pi = live ? C.pos[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float inv_s2 = 1.0f / (p.sigma * p.sigma);
  const float inv2s2 = 0.5f * inv_s2;
  const float scale = INV_SQRT_2PI / p.sigma * inv_s2;
  const bool recur = p.bin <= 2.0f * p.sigma;
  const unsigned below = (1u << lane) - 1u;
  float g[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
  auto flush = [&](int count) {
    if (lane < count) {
      const float4 v = q_v[warp][lane];
      float psi = 0.f;
      gauss_bins(p, v.w, inv2s2, recur, [&](int b, float x, float G) { psi = fmaf(sh_w[b] * x, G, psi); });
      const float sc = psi * scale / v.w;
      q_v[warp][lane] = make_float4(sc * v.x, sc * v.y, sc * v.z, 0.f);
    }
    __syncwarp();
    float part[3] = {0.f, 0.f, 0.f};
    for (int e = 0; e < count; ++e)
      if (q_o[warp][e] == lane) {
        const float4 v = q_v[warp][e];
        part[0] += v.x;
        part[1] += v.y;
        part[2] += v.z;
      }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float y = __fsub_rn(part[d], c[d]), t = __fadd_rn(g[d], y);
      c[d] = __fsub_rn(__fsub_rn(t, g[d]), y);
      g[d] = t;
    }
  };
  int qn = 0;
  for (int off = 0; off < 27; ++off) {
    const int nb = live ? neighbour_cell(C, pi, off) : 0;
    const int cs = live ? C.start[nb] : 0, len = live ? C.start[nb + 1] - cs : 0;
    const int maxlen = __reduce_max_sync(0xffffffffu, len);
    for (int k = 0; k < maxlen; ++k) {
      bool in = false;
      float dx = 0.f, dy = 0.f, dz = 0.f, r2 = 0.f;
      if (k < len) {
        const int j = C.order[cs + k];
        const float4 pj = C.pos[cs + k];
        dx = min_image(pi.x - pj.x, p.box.x, p.inv_box.x);
        dy = min_image(pi.y - pj.y, p.box.y, p.inv_box.y);
        dz = min_image(pi.z - pj.z, p.box.z, p.inv_box.z);
        r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        in = j != i && r2 < p.cut2 && r2 > 0.f;
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int pos = qn + __popc(m & below);
        q_v[warp][pos] = make_float4(dx, dy, dz, sqrtf(r2));
        q_o[warp][pos] = (unsigned char)lane;
      }
      qn += __popc(m);
      if (qn >= 32) {
        __syncwarp();
        flush(32);
        __syncwarp();
        if (lane < qn - 32) {
          q_v[warp][lane] = q_v[warp][32 + lane];
          q_o[warp][lane] = q_o[warp][32 + lane];
        }
        __syncwarp();
        qn -= 32;
      }
    }
  }
  __syncwarp();
  flush(qn);
  if (live) {
    float* out = p.grad + ((int64_t)frame * p.lst.n + i) * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) out[d] = __fsub_rn(g[d], c[d]);
  }
}

// ---------------------------------------------------------------------------
// structure-factor adjoint
// ---------------------------------------------------------------------------
__device__ __forceinline__ void phase_sc(int32_t ph, float* s, float* c) {
  sincospif(__fmul_rn((float)ph, 9.313225746154785e-10f), s, c);  // ph * 2^-31 turns
}

__device__ __forceinline__ void kahan3(float (&acc)[3], float (&cmp)[3], const float (&v)[3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float y = __fsub_rn(v[d], cmp[d]), t = __fadd_rn(acc[d], y);
    cmp[d] = __fsub_rn(__fsub_rn(t, acc[d]), y);
    acc[d] = t;
  }
}

// c[f][slot(k)] = u_k conj(rho[f][k]); holes of the slot table stay zero
__global__ void sk_coef_kernel(const float2* __restrict__ rho, int32_t n_k, int32_t n_frames,
                               const int32_t* __restrict__ slot, const float* __restrict__ u,
                               int64_t n_slots, float2* __restrict__ coef) {
  const int64_t total = (int64_t)n_frames * n_k;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int f = (int)(i / n_k), k = (int)(i % n_k);
    const float2 r = rho[i];
    const float w = u[k];
    coef[(int64_t)f * n_slots + slot[k]] = make_float2(w * r.x, -w * r.y);
  }
}

struct SkColumn {
  int32_t nx, ny, nz0, len;
};
struct SkChunk {
  int32_t col0, col1, slot0, slot1;  // columns col0..col1-1 use slots slot0..slot1-1
};

constexpr int SKC_THREADS = 256;
constexpr int SKC_APT = 4;                           // atoms per thread
constexpr int SKC_ATOMS = SKC_THREADS * SKC_APT;     // atoms per block
constexpr int SKC_SLOTS = 2048;                      // coefficient slots per chunk
constexpr int SKC_COLS = 512;                        // columns per chunk
constexpr int SKC_ANCHOR = 64;                       // exact re-anchoring interval along nz

__global__ void __launch_bounds__(SKC_THREADS)
    sk_adjoint_columns_kernel(const int4* __restrict__ fx /*[F][n]*/, int32_t n,
                              const SkColumn* __restrict__ cols, const SkChunk* __restrict__ chunks,
                              int32_t n_chunks, const float2* __restrict__ coef, int64_t n_slots,
                              float scale, float* __restrict__ grad /*[F][n][3]*/) {
  __shared__ float2 s_c[SKC_SLOTS];
  __shared__ SkColumn s_col[SKC_COLS];
  const int f = blockIdx.y;
  const float2* C = coef + (int64_t)f * n_slots;
  int4 q[SKC_APT];
  float zc[SKC_APT], zs[SKC_APT];
  float acc[SKC_APT][3], cmp[SKC_APT][3];
#pragma unroll
  for (int a = 0; a < SKC_APT; ++a) {
    const int i = blockIdx.x * SKC_ATOMS + a * SKC_THREADS + threadIdx.x;
    q[a] = i < n ? fx[(int64_t)f * n + i] : make_int4(0, 0, 0, 0);
    phase_sc(q[a].z, &zs[a], &zc[a]);
#pragma unroll
    for (int d = 0; d < 3; ++d) acc[a][d] = cmp[a][d] = 0.f;
  }
  for (int ch = 0; ch < n_chunks; ++ch) {
    const SkChunk K = chunks[ch];
    __syncthreads();
    for (int t = threadIdx.x; t < K.slot1 - K.slot0; t += SKC_THREADS) s_c[t] = C[K.slot0 + t];
    for (int t = threadIdx.x; t < K.col1 - K.col0; t += SKC_THREADS) s_col[t] = cols[K.col0 + t];
    __syncthreads();
    float part[SKC_APT][3];
#pragma unroll
    for (int a = 0; a < SKC_APT; ++a) part[a][0] = part[a][1] = part[a][2] = 0.f;
    int slot = 0;
    for (int c = 0; c < K.col1 - K.col0; ++c) {
      const SkColumn col = s_col[c];
      float s0[SKC_APT], sz[SKC_APT];
#pragma unroll
      for (int a = 0; a < SKC_APT; ++a) s0[a] = sz[a] = 0.f;
      for (int m0 = 0; m0 < col.len; m0 += SKC_ANCHOR) {
        const int m1 = min(col.len, m0 + SKC_ANCHOR);
        float er[SKC_APT], ei[SKC_APT];
#pragma unroll
        for (int a = 0; a < SKC_APT; ++a) {
          const int32_t ph = (int32_t)((uint32_t)col.nx * (uint32_t)q[a].x + (uint32_t)col.ny * (uint32_t)q[a].y +
                                       (uint32_t)(col.nz0 + m0) * (uint32_t)q[a].z);
          phase_sc(ph, &ei[a], &er[a]);
        }
        float nz = (float)(col.nz0 + m0);
#pragma unroll 4
        for (int m = m0; m < m1; ++m) {
          const float2 cc = s_c[slot + m];
#pragma unroll
          for (int a = 0; a < SKC_APT; ++a) {
            const float im = fmaf(cc.x, ei[a], cc.y * er[a]);  // Im(c e)
            s0[a] += im;
            sz[a] = fmaf(nz, im, sz[a]);
            const float nr = fmaf(er[a], zc[a], -ei[a] * zs[a]);
            ei[a] = fmaf(er[a], zs[a], ei[a] * zc[a]);
            er[a] = nr;
          }
          nz += 1.0f;
        }
      }
      slot += col.len;
      const float fxn = (float)col.nx, fyn = (float)col.ny;
#pragma unroll
      for (int a = 0; a < SKC_APT; ++a) {
        part[a][0] = fmaf(fxn, s0[a], part[a][0]);
        part[a][1] = fmaf(fyn, s0[a], part[a][1]);
        part[a][2] += sz[a];
      }
    }
#pragma unroll
    for (int a = 0; a < SKC_APT; ++a) kahan3(acc[a], cmp[a], part[a]);
  }
#pragma unroll
  for (int a = 0; a < SKC_APT; ++a) {
    const int i = blockIdx.x * SKC_ATOMS + a * SKC_THREADS + threadIdx.x;
    if (i >= n) continue;
    float* g = grad + ((int64_t)f * n + i) * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = -scale * __fsub_rn(acc[a][d], cmp[a][d]);
  }
}

constexpr int SKD_THREADS = 256;
constexpr int SKD_KT = 512;

// arbitrary vectors: one exact phase per (atom, vector); coef in vector order
__global__ void __launch_bounds__(SKD_THREADS)
    sk_adjoint_direct_kernel(const int4* __restrict__ fx, int32_t n, const int4* __restrict__ kv,
                             int32_t n_k, const float2* __restrict__ coef, float scale,
                             float* __restrict__ grad) {
  __shared__ int4 s_k[SKD_KT];
  __shared__ float2 s_c[SKD_KT];
  const int f = blockIdx.y;
  const int i = blockIdx.x * SKD_THREADS + threadIdx.x;
  const bool live = i < n;
  const int4 q = live ? fx[(int64_t)f * n + i] : make_int4(0, 0, 0, 0);
  const float2* C = coef + (int64_t)f * n_k;
  float acc[3] = {0.f, 0.f, 0.f}, cmp[3] = {0.f, 0.f, 0.f};
  for (int k0 = 0; k0 < n_k; k0 += SKD_KT) {
    const int nk = min(SKD_KT, n_k - k0);
    __syncthreads();
    for (int t = threadIdx.x; t < nk; t += SKD_THREADS) {
      s_k[t] = kv[k0 + t];
      s_c[t] = C[k0 + t];
    }
    __syncthreads();
    if (!live) continue;
    float part[3] = {0.f, 0.f, 0.f};
    for (int t = 0; t < nk; ++t) {
      const int4 n4 = s_k[t];
      const int32_t ph = (int32_t)((uint32_t)n4.x * (uint32_t)q.x + (uint32_t)n4.y * (uint32_t)q.y +
                                   (uint32_t)n4.z * (uint32_t)q.z);
      float sn, cs;
      phase_sc(ph, &sn, &cs);
      const float2 cc = s_c[t];
      const float im = fmaf(cc.x, sn, cc.y * cs);
      part[0] = fmaf(im, (float)n4.x, part[0]);
      part[1] = fmaf(im, (float)n4.y, part[1]);
      part[2] = fmaf(im, (float)n4.z, part[2]);
    }
    kahan3(acc, cmp, part);
  }
  if (live) {
    float* g = grad + ((int64_t)f * n + i) * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = -scale * __fsub_rn(acc[d], cmp[d]);
  }
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
// column plan of a vector list: columns of consecutive nz at fixed (nx, ny),
// holes inside a column get zero coefficients; chunks sized for shared memory
struct SkColumnsPlan {
  std::vector<SkColumn> cols;
  std::vector<SkChunk> chunks;
  std::vector<int32_t> slot;  // [n_k]
  int64_t n_slots = 0;
  bool duplicates = false;
};

static SkColumnsPlan build_columns(const std::vector<int32_t>& kvec) {
  const int n_k = (int)(kvec.size() / 3);
  std::vector<int32_t> order(n_k);
  for (int k = 0; k < n_k; ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    const int32_t* A = &kvec[3 * (size_t)a];
    const int32_t* B = &kvec[3 * (size_t)b];
    if (A[0] != B[0]) return A[0] < B[0];
    if (A[1] != B[1]) return A[1] < B[1];
    if (A[2] != B[2]) return A[2] < B[2];
    return a < b;
  });
  SkColumnsPlan P;
  P.slot.assign(n_k, -1);
  auto K = [&](int t, int c) { return kvec[3 * (size_t)order[t] + c]; };
  int64_t slot = 0;
  for (int s = 0; s < n_k;) {
    const int32_t nx = K(s, 0), ny = K(s, 1);
    int e = s;
    while (e < n_k && K(e, 0) == nx && K(e, 1) == ny) ++e;
    // split the (nx, ny) group where nz jumps by more than 8 or the column
    // would outgrow a chunk
    int a = s;
    while (a < e) {
      const int32_t nz0 = K(a, 2);
      int b = a + 1;
      while (b < e && K(b, 2) - K(b - 1, 2) <= 8 && K(b, 2) - nz0 < SKC_SLOTS) ++b;
      for (int t = a; t < b; ++t) {
        if (t > a && K(t, 2) == K(t - 1, 2)) P.duplicates = true;
        P.slot[order[t]] = (int32_t)(slot + (K(t, 2) - nz0));
      }
      const int32_t len = K(b - 1, 2) - nz0 + 1;
      P.cols.push_back(SkColumn{nx, ny, nz0, len});
      slot += len;
      a = b;
    }
    s = e;
  }
  P.n_slots = slot;
  // chunks: consecutive columns, <= SKC_SLOTS slots and <= SKC_COLS columns each
  int64_t s0 = 0, cur = 0;
  int c0 = 0;
  for (int c = 0; c < (int)P.cols.size(); ++c) {
    const int len = P.cols[c].len;
    if (c > c0 && (cur + len > SKC_SLOTS || c - c0 >= SKC_COLS)) {
      P.chunks.push_back(SkChunk{c0, c, (int32_t)s0, (int32_t)(s0 + cur)});
      s0 += cur;
      cur = 0;
      c0 = c;
    }
    cur += len;
  }
  if (!P.cols.empty()) P.chunks.push_back(SkChunk{c0, (int32_t)P.cols.size(), (int32_t)s0, (int32_t)(s0 + cur)});
  return P;
}

// device tables of the S(k) adjoint for one vector list: the column plan
// (when the columns average >= 8 vectors and holes are few) or the vectors
// themselves; lattice densities keep theirs per lattice
struct SkAdjointPlan {
  bool columns = false;
  int64_t n_slots = 0;
  int32_t n_chunks = 0;
  DevBuf<SkColumn> cols;
  DevBuf<SkChunk> chunks;
  DevBuf<int32_t> slot;
  DevBuf<int4> kv;
};

void sk_adjoint_plans_free(amdat_ctx* ctx) {
  for (auto& kv : ctx->sk_adjoint_plans) delete kv.second;
  ctx->sk_adjoint_plans.clear();
}

static SkAdjointPlan* sk_adjoint_plan_build(const std::vector<int32_t>& kvec) {
  const int nk = (int)(kvec.size() / 3);
  auto* A = new SkAdjointPlan();
  try {
    SkColumnsPlan plan = build_columns(kvec);
    A->columns = !plan.duplicates && plan.n_slots <= 2 * (int64_t)nk && (double)nk >= 8.0 * (double)plan.cols.size();
    A->slot.reserve(std::max(nk, 1));
    if (A->columns) {
      A->n_slots = plan.n_slots;
      A->n_chunks = (int32_t)plan.chunks.size();
      A->cols.reserve(std::max<size_t>(plan.cols.size(), 1));
      A->chunks.reserve(std::max<size_t>(plan.chunks.size(), 1));
      AMDAT_CUDA(cudaMemcpy(A->cols.ptr, plan.cols.data(), plan.cols.size() * sizeof(SkColumn), cudaMemcpyHostToDevice));
      AMDAT_CUDA(cudaMemcpy(A->chunks.ptr, plan.chunks.data(), plan.chunks.size() * sizeof(SkChunk), cudaMemcpyHostToDevice));
      AMDAT_CUDA(cudaMemcpy(A->slot.ptr, plan.slot.data(), (size_t)nk * 4, cudaMemcpyHostToDevice));
    } else {
      A->n_slots = nk;
      std::vector<int32_t> slot(nk);
      std::vector<int4> hk(nk);
      for (int k = 0; k < nk; ++k) {
        slot[k] = k;
        hk[k] = make_int4(kvec[3 * (size_t)k], kvec[3 * (size_t)k + 1], kvec[3 * (size_t)k + 2], 0);
      }
      A->kv.reserve(std::max(nk, 1));
      AMDAT_CUDA(cudaMemcpy(A->kv.ptr, hk.data(), (size_t)nk * sizeof(int4), cudaMemcpyHostToDevice));
      AMDAT_CUDA(cudaMemcpy(A->slot.ptr, slot.data(), (size_t)nk * 4, cudaMemcpyHostToDevice));
    }
  } catch (...) {
    delete A;
    throw;
  }
  return A;
}

static void sg_check(amdat_ctx* ctx, const int32_t* frames, int32_t n_frames, float sigma, float r_max,
                     int32_t n_bins) {
  if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
  AMDAT_REQUIRE(frames != nullptr && n_frames >= 1 && n_frames <= 65535, "need 1..65535 frames");
  for (int f = 0; f < n_frames; ++f)
    AMDAT_REQUIRE(frames[f] >= 0 && frames[f] < ctx->n_frames, "frame index out of range");
  AMDAT_REQUIRE(sigma > 0.0f && r_max > 0.0f, "sigma and r_max must be positive");
  AMDAT_REQUIRE(n_bins >= 1 && n_bins <= 4096, "n_bins must be in [1, 4096]");
  const float half = 0.5f * std::min(ctx->box[0], std::min(ctx->box[1], ctx->box[2]));
  AMDAT_REQUIRE(r_max + SG_CUT * sigma <= half, "r_max + 6 sigma must not exceed half the box");
  const float bin = r_max / (float)n_bins;
  AMDAT_REQUIRE(SG_CUT * sigma / bin <= 256.0f, "sigma spans more than 256 bins");
}

static SGParams sg_params(amdat_ctx* ctx, const ListEntry& e, const int32_t* d_frames, float sigma,
                          float r_max, int32_t n_bins) {
  SGParams p{};
  p.w = ctx->w.ptr;
  p.n_pad = ctx->n_pad;
  p.lst = sglist(e);
  p.frames = d_frames;
  p.box = make_float3(ctx->box[0], ctx->box[1], ctx->box[2]);
  p.inv_box = make_float3(1.0f / ctx->box[0], 1.0f / ctx->box[1], 1.0f / ctx->box[2]);
  p.sigma = sigma;
  p.bin = r_max / (float)n_bins;
  const float cut = r_max + SG_CUT * sigma;
  p.cut2 = cut * cut;
  p.n_bins = n_bins;
  p.span = (int)std::ceil(SG_CUT * sigma / p.bin);
  return p;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// cell grid for a cutoff: used when every axis holds at least three cells
// (cell edge >= cutoff) and the list is large enough to gain from it
static bool cell_grid(amdat_ctx* ctx, const ListEntry& e, float cut, int3& nc) {
  nc = make_int3((int)std::floor(ctx->box[0] / cut), (int)std::floor(ctx->box[1] / cut),
                 (int)std::floor(ctx->box[2] / cut));
  const int64_t cells = (int64_t)nc.x * nc.y * nc.z;
  return e.n >= 1024 && nc.x >= 3 && nc.y >= 3 && nc.z >= 3 && cells <= (1 << 22);
}

// builds one frame's cell lists in ctx->scratch2 and returns their view
static SGCells build_cells(amdat_ctx* ctx, const ListEntry& e, int32_t frame, int3 nc) {
  const int n = e.n, n_cells = nc.x * nc.y * nc.z;
  size_t o = 0;
  const size_t o_cell = o; o = align256(o + (size_t)n * 4);
  const size_t o_cnt = o; o = align256(o + (size_t)n_cells * 4);
  const size_t o_start = o; o = align256(o + (size_t)(n_cells + 1) * 4);
  const size_t o_cur = o; o = align256(o + (size_t)n_cells * 4);
  const size_t o_ord = o; o = align256(o + (size_t)n * 4);
  const size_t o_pos = o; o = align256(o + (size_t)n * sizeof(float4));
  unsigned char* b = ctx->scratch2.reserve(o);
  const float* P = ctx->w.ptr + (int64_t)frame * 3 * ctx->n_pad;
  SGCells C;
  C.nc = nc;
  C.lo = make_float3(ctx->box_lo[0], ctx->box_lo[1], ctx->box_lo[2]);
  C.inv_cell = make_float3((float)nc.x / ctx->box[0], (float)nc.y / ctx->box[1], (float)nc.z / ctx->box[2]);
  C.start = (const int32_t*)(b + o_start);
  C.order = (const int32_t*)(b + o_ord);
  C.pos = (const float4*)(b + o_pos);
  cudaStream_t st = ctx->stream;
  AMDAT_CUDA(cudaMemsetAsync(b + o_cnt, 0, (size_t)n_cells * 4, st));
  const unsigned gn = (unsigned)ceil_div(n, 256), gc = (unsigned)ceil_div(n_cells, 256);
  cell_assign_kernel<<<gn, 256, 0, st>>>(P, ctx->n_pad, sglist(e), C.lo, C.inv_cell, nc, (int32_t*)(b + o_cell),
                                         (int32_t*)(b + o_cnt));
  cell_scan_kernel<<<1, 1024, 0, st>>>((const int32_t*)(b + o_cnt), n_cells, (int32_t*)(b + o_start),
                                       (int32_t*)(b + o_cur));
  cell_scatter_kernel<<<gn, 256, 0, st>>>((const int32_t*)(b + o_cell), n, (int32_t*)(b + o_cur),
                                          (int32_t*)(b + o_ord));
  cell_sort_kernel<<<gc, 256, 0, st>>>((const int32_t*)(b + o_start), n_cells, (int32_t*)(b + o_ord), P,
                                       ctx->n_pad, sglist(e), (float4*)(b + o_pos));
  check_launch("cell lists");
  count_launch(ctx, 4);
  return C;
}

// dynamic shared memory beyond what fits beside the static arrays under the
// default 48 KB needs the opt-in attribute
static void set_smem(const void* fn, size_t shm) {
  if (shm > 32 * 1024)
    AMDAT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_gsmooth_run(amdat_ctx* ctx, int32_t list, const int32_t* frames, int32_t n_frames,
                               float sigma, float r_max, int32_t n_bins, int32_t out_flags,
                               double* h) {
  return guarded([&] {
    check_ctx(ctx);
    sg_check(ctx, frames, n_frames, sigma, r_max, n_bins);
    AMDAT_REQUIRE(h != nullptr, "null output");
    const ListEntry& e = list_entry(ctx, list);
    const bool dev = out_flags == AMDAT_OUT_DEVICE;
    const size_t o_h = align256((size_t)n_frames * 4);
    unsigned char* base = ctx->scratch.reserve(o_h + (size_t)n_bins * 8);
    int32_t* d_frames = (int32_t*)base;
    double* d_h = dev ? h : (double*)(base + o_h);
    AMDAT_CUDA(cudaMemcpyAsync(d_frames, frames, n_frames * 4, cudaMemcpyHostToDevice, ctx->stream));
    AMDAT_CUDA(cudaMemsetAsync(d_h, 0, (size_t)n_bins * 8, ctx->stream));
    if (e.n > 1) {
      SGParams p = sg_params(ctx, e, d_frames, sigma, r_max, n_bins);
      p.h = d_h;
      // fixed-point scale: a block's bin collects at most SG_THREADS * n terms
      // of at most 1/(sqrt(2 pi) sigma); keep that below 2^62
      const double bound = (double)SG_THREADS * (double)e.n * (double)INV_SQRT_2PI / (double)sigma;
      const float qscale = (float)std::ldexp(1.0, (int)std::floor(std::log2(std::ldexp(1.0, 62) / bound)));
      const size_t shm = (size_t)n_bins * 8;
      int3 nc;
      if (cell_grid(ctx, e, std::sqrt(p.cut2), nc)) {
        set_smem((const void*)gsmooth_cells_kernel, shm);
        for (int f = 0; f < n_frames; ++f) {
          const SGCells C = build_cells(ctx, e, frames[f], nc);
          KernelTimer kt(ctx, "gsmooth_kernel");
          gsmooth_cells_kernel<<<(unsigned)ceil_div(e.n, SG_THREADS), SG_THREADS, shm, ctx->stream>>>(p, C, qscale);
          check_launch("gsmooth_cells_kernel");
          count_launch(ctx);
        }
      } else {
        set_smem((const void*)gsmooth_kernel, shm);
        dim3 grid((unsigned)ceil_div(e.n, SG_THREADS), (unsigned)n_frames);
        KernelTimer kt(ctx, "gsmooth_kernel");
        gsmooth_kernel<<<grid, SG_THREADS, shm, ctx->stream>>>(p, qscale);
        check_launch("gsmooth_kernel");
        count_launch(ctx);
      }
    }
    if (!dev) AMDAT_CUDA(cudaMemcpyAsync(h, d_h, (size_t)n_bins * 8, cudaMemcpyDeviceToHost, ctx->stream));
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

amdat_status amdat_gsmooth_adjoint(amdat_ctx* ctx, int32_t list, const int32_t* frames,
                                   int32_t n_frames, float sigma, float r_max, int32_t n_bins,
                                   const double* dl_dh, int32_t io_flags, float* grad) {
  return guarded([&] {
    check_ctx(ctx);
    sg_check(ctx, frames, n_frames, sigma, r_max, n_bins);
    AMDAT_REQUIRE(dl_dh != nullptr && grad != nullptr, "null argument");
    const ListEntry& e = list_entry(ctx, list);
    const size_t gbytes = (size_t)n_frames * e.n * 3 * sizeof(float);
    const size_t o_w = align256((size_t)n_frames * 4), o_g = align256(o_w + (size_t)n_bins * 8);
    const bool dev = io_flags == AMDAT_OUT_DEVICE;
    unsigned char* base = ctx->scratch.reserve(o_g + (dev ? 0 : gbytes));
    int32_t* d_frames = (int32_t*)base;
    double* d_w = (double*)(base + o_w);
    float* d_g = dev ? grad : (float*)(base + o_g);
    AMDAT_CUDA(cudaMemcpyAsync(d_frames, frames, n_frames * 4, cudaMemcpyHostToDevice, ctx->stream));
    AMDAT_CUDA(cudaMemcpyAsync(d_w, dl_dh, (size_t)n_bins * 8,
                               dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
    if (e.n > 0) {
      SGParams p = sg_params(ctx, e, d_frames, sigma, r_max, n_bins);
      p.wgt = d_w;
      p.grad = d_g;
      const size_t shm = (size_t)n_bins * 4;
      int3 nc;
      if (cell_grid(ctx, e, std::sqrt(p.cut2), nc)) {
        set_smem((const void*)gsmooth_cells_adjoint_kernel, shm);
        for (int f = 0; f < n_frames; ++f) {
          const SGCells C = build_cells(ctx, e, frames[f], nc);
          KernelTimer kt(ctx, "gsmooth_adjoint_kernel");
          gsmooth_cells_adjoint_kernel<<<(unsigned)ceil_div(e.n, SG_THREADS), SG_THREADS, shm, ctx->stream>>>(
              p, C, f);
          check_launch("gsmooth_cells_adjoint_kernel");
          count_launch(ctx);
        }
      } else {
        set_smem((const void*)gsmooth_adjoint_kernel, shm);
        dim3 grid((unsigned)ceil_div(e.n, SG_THREADS), (unsigned)n_frames);
        KernelTimer kt(ctx, "gsmooth_adjoint_kernel");
        gsmooth_adjoint_kernel<<<grid, SG_THREADS, shm, ctx->stream>>>(p);
        check_launch("gsmooth_adjoint_kernel");
        count_launch(ctx);
      }
    }
    if (!dev && gbytes) AMDAT_CUDA(cudaMemcpyAsync(grad, d_g, gbytes, cudaMemcpyDeviceToHost, ctx->stream));
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

amdat_status amdat_structure_factor_adjoint(amdat_ctx* ctx, int32_t density_handle,
                                            const int32_t* shell_offsets, int32_t n_shells,
                                            const double* dl_ds, int32_t io_flags, float* grad) {
  return guarded([&] {
    check_ctx(ctx);
    Density& d = density(ctx, density_handle);
    AMDAT_REQUIRE(shell_offsets != nullptr && n_shells >= 1, "need >= 1 shell");
    AMDAT_REQUIRE(shell_offsets[0] >= 0 && shell_offsets[n_shells] <= d.n_k, "shells outside the density");
    AMDAT_REQUIRE(dl_ds != nullptr && grad != nullptr, "null argument");
    AMDAT_REQUIRE(d.period > 0.0f, "density has no period");
    for (int s = 0; s < n_shells; ++s)
      AMDAT_REQUIRE(shell_offsets[s] <= shell_offsets[s + 1], "shell offsets must ascend");
    const bool dev = io_flags == AMDAT_OUT_DEVICE;
    const ListEntry& e = list_entry(ctx, d.list);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(e.n == d.n_list, "the density's list changed size since the density was computed");
    for (int f = 0; f < d.n_frames; ++f)
      AMDAT_REQUIRE(d.frames[f] < ctx->n_frames, "the density's frames are not in the current trajectory");
    const int F = d.n_frames, n = e.n, nk = d.n_k;
    const size_t gbytes = (size_t)F * n * 3 * sizeof(float);
    // per-vector weights u_k = 2 w_s / H_s (zero outside the shells)
    std::vector<double> w(n_shells);
    if (dev)
      AMDAT_CUDA(cudaMemcpy(w.data(), dl_ds, (size_t)n_shells * 8, cudaMemcpyDeviceToHost));
    else
      std::memcpy(w.data(), dl_ds, (size_t)n_shells * 8);
    std::vector<float> u(std::max(nk, 1), 0.f);
    for (int s = 0; s < n_shells; ++s) {
      const int cnt = shell_offsets[s + 1] - shell_offsets[s];
      for (int k = shell_offsets[s]; k < shell_offsets[s + 1]; ++k) u[k] = (float)(2.0 * w[s] / cnt);
    }
    if (n == 0 || nk == 0) {
      if (gbytes) {
        if (dev) AMDAT_CUDA(cudaMemsetAsync(grad, 0, gbytes, ctx->stream));
        else std::memset(grad, 0, gbytes);
      }
      AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
      return;
    }
    // lattice densities on compute capability 10.x: the tensor-core adjoint
    // (AMDAT_SK_ADJOINT=columns selects the FP32 column kernel instead)
    const char* sel = std::getenv("AMDAT_SK_ADJOINT");
    if (!d.lattice_key.empty() && tc_enabled(ctx) && !(sel && std::strcmp(sel, "columns") == 0)) {
      TcPlan* tp = lattice_tc_plan(ctx, d.lattice_key);
      float max_u = 0.f;
      for (int k = 0; k < nk; ++k) max_u = std::max(max_u, std::fabs(u[k]));
      const size_t o_fr = 0, o_u = align256((size_t)F * 4), o_fx = align256(o_u + (size_t)nk * 4);
      const size_t o_g = align256(o_fx + (size_t)F * n * sizeof(int4));
      unsigned char* base = ctx->scratch.reserve(o_g + (dev ? 0 : gbytes));
      cudaStream_t st = ctx->stream;
      AMDAT_CUDA(cudaMemcpyAsync(base + o_fr, d.frames.data(), (size_t)F * 4, cudaMemcpyHostToDevice, st));
      AMDAT_CUDA(cudaMemcpyAsync(base + o_u, u.data(), (size_t)nk * 4, cudaMemcpyHostToDevice, st));
      fixed_turns_launch(ctx, (const int32_t*)(base + o_fr), F, e, d.period, (int4*)(base + o_fx));
      float* d_g = dev ? grad : (float*)(base + o_g);
      sk_adjoint_tc_run(ctx, *tp, (const int4*)(base + o_fx), n, F, d.rho->ptr, nk, (const float*)(base + o_u),
                        max_u, d.period, d_g);
      if (!dev) AMDAT_CUDA(cudaMemcpyAsync(grad, d_g, gbytes, cudaMemcpyDeviceToHost, st));
      AMDAT_CUDA(cudaStreamSynchronize(st));
      return;
    }
    // the adjoint plan: kept per lattice, built per call for explicit lists
    std::unique_ptr<SkAdjointPlan> own;
    SkAdjointPlan* A = nullptr;
    if (!d.lattice_key.empty()) {
      auto it = ctx->sk_adjoint_plans.find(d.lattice_key);
      if (it == ctx->sk_adjoint_plans.end())
        it = ctx->sk_adjoint_plans.emplace(d.lattice_key, sk_adjoint_plan_build(d.kvec)).first;
      A = it->second;
    } else {
      own.reset(sk_adjoint_plan_build(d.kvec));
      A = own.get();
    }
    const int64_t n_slots = A->n_slots;
    size_t o = 0;
    const size_t o_fr = o; o = align256(o + (size_t)F * 4);
    const size_t o_u = o; o = align256(o + (size_t)nk * 4);
    const size_t o_fx = o; o = align256(o + (size_t)F * n * sizeof(int4));
    const size_t o_c = o; o = align256(o + (size_t)F * n_slots * sizeof(float2));
    const size_t o_g = o; o = align256(o + (dev ? 0 : gbytes));
    unsigned char* base = ctx->scratch.reserve(o);
    cudaStream_t st = ctx->stream;
    AMDAT_CUDA(cudaMemcpyAsync(base + o_fr, d.frames.data(), (size_t)F * 4, cudaMemcpyHostToDevice, st));
    AMDAT_CUDA(cudaMemcpyAsync(base + o_u, u.data(), (size_t)nk * 4, cudaMemcpyHostToDevice, st));
    float2* coef = (float2*)(base + o_c);
    if (A->columns) AMDAT_CUDA(cudaMemsetAsync(coef, 0, (size_t)F * n_slots * sizeof(float2), st));
    const int64_t tot = (int64_t)F * nk;
    sk_coef_kernel<<<(unsigned)std::min<int64_t>(ceil_div(tot, 256), (int64_t)ctx->n_sm * 16), 256, 0, st>>>(
        d.rho->ptr, nk, F, A->slot.ptr, (const float*)(base + o_u), n_slots, coef);
    check_launch("sk_coef_kernel");
    count_launch(ctx);
    fixed_turns_launch(ctx, (const int32_t*)(base + o_fr), F, e, d.period, (int4*)(base + o_fx));
    float* d_g = dev ? grad : (float*)(base + o_g);
    const float scale = (float)(6.283185307179586476925286766559 / (double)d.period);
    if (A->columns) {
      dim3 grid((unsigned)ceil_div(n, SKC_ATOMS), (unsigned)F);
      KernelTimer kt(ctx, "sk_adjoint_columns_kernel");
      sk_adjoint_columns_kernel<<<grid, SKC_THREADS, 0, st>>>((const int4*)(base + o_fx), n, A->cols.ptr,
                                                              A->chunks.ptr, A->n_chunks, coef, n_slots,
                                                              scale, d_g);
      check_launch("sk_adjoint_columns_kernel");
    } else {
      dim3 grid((unsigned)ceil_div(n, SKD_THREADS), (unsigned)F);
      KernelTimer kt(ctx, "sk_adjoint_direct_kernel");
      sk_adjoint_direct_kernel<<<grid, SKD_THREADS, 0, st>>>((const int4*)(base + o_fx), n, A->kv.ptr, nk,
                                                             coef, scale, d_g);
      check_launch("sk_adjoint_direct_kernel");
    }
    count_launch(ctx);
    if (!dev) AMDAT_CUDA(cudaMemcpyAsync(grad, d_g, gbytes, cudaMemcpyDeviceToHost, st));
    AMDAT_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
