// Spatially binned displacement analyses:
//   System::boxify                      (src/system.cpp:4799-4870)
//   Trajectory_List_Bins::assign_bins   (src/trajectory_list_bins.cpp:949-1096),
//     with the region rules of its constructors (:207-394)
//   Bin_Static_Analysis::analyze        (src/bin_static_analysis.h:69-111): one
//     analysis per bin over the list members in that bin at the start frame t0
//   Bin_Dynamics_Analysis::list_displacementkernel (src/bin_dynamics_analysis.h):
//     the members in the bin at both t0 and t1 (persistence), with the pairs of
//     displacement_list(this), i.e. fullblock 0
// for the MSD and NGP moments (Mean_Square_Displacement / Non_Gaussian_Parameter
// listkernels) and F_s
// (Incoherent_Scattering_Function::listkernel) of every bin at once.
//
// The reference builds one time-dependent list per bin and runs the analysis
// B times.  Here a bin map (flat bin per atom per frame, int32, -1 outside)
// is built once on the device, and one pass over (time pair, list member)
// keys each term by the member's bin: every atom's trajectory is read once per
// pair for all bins together.  Terms of one warp that share a bin are summed
// by the warp's lowest such lane (FP64, lane order) and added with one atomic to
// a per-block shared-memory accumulator [bin][stride] (|dr|^2, |dr|^4 when
// asked for, the shell means), flushed to the global [bin][gap][stride] sums at
// the end of each item.  Counts are
// exact integers; the FP64 sums are order-independent to rounding (atomics).
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

#include "disp_common.cuh"
#include "engine.h"

namespace amdat {

constexpr int BN_THREADS = 256;
constexpr int BN_CHUNK = 2048;
constexpr int BN_MAX_FS = 8;
constexpr size_t BN_STAGE_LIMIT = 48 * 1024;  // shared accumulators per block
constexpr int BN_WARPS = BN_THREADS / 32;
constexpr int BN_SUM_CHUNK = 8192;                 // members per item of the sums kernel
constexpr size_t BN_SUM_SMEM_LIMIT = 96 * 1024;   // its per-warp accumulators

// --- boxify and bin assignment -------------------------------------------------
__global__ void boxify_kernel(float* __restrict__ w, int64_t n_pad, int32_t n_atoms, int64_t n_terms,
                              float3 lo, float3 hi) {
  const float L[3] = {__fsub_rn(hi.x, lo.x), __fsub_rn(hi.y, lo.y), __fsub_rn(hi.z, lo.z)};
  const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_terms;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = i / n_atoms, a = i - t * n_atoms;
    float* c = w + t * 3 * n_pad + a;
    const float x[3] = {c[0], c[n_pad], c[2 * n_pad]};
    bool out = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) out |= (x[d] < l[d]) | (x[d] > h[d]);
    if (!out) continue;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float sh = x[d] > h[d] ? -1.f : (x[d] < l[d] ? 1.f : 0.f);
      c[d * n_pad] = __fadd_rn(x[d], __fmul_rn(L[d], sh));
    }
  }
}

// int((x - lo + 10 FLT_EPSILON) / (hi - lo + 20 FLT_EPSILON) * n): the two
// differences in FP32, everything after them in FP64
__device__ __forceinline__ int bin_axis(float x, float lo, float hi, int n) {
  const double num = __dadd_rn((double)__fsub_rn(x, lo), (double)FLT_EPSILON * 10.0);
  const double den = __dadd_rn((double)__fsub_rn(hi, lo), (double)FLT_EPSILON * 20.0);
  return (int)__dmul_rn(__ddiv_rn(num, den), (double)(float)n);
}

// --- distance bins (Trajectory_List_Bins distance constructors) -------------
// The reference's FP32 chains, operation by operation (see amdat_bins_distance):
// Coordinate::vector_unwrapped + length (src/coordinate.cpp:98-124,
// src/coordinate.h:55) to the nearest member of another list, the minimum-image
// distance to a point, or the distance to a plane.
constexpr int BD_THREADS = 256;
constexpr int BD_TILE = 1024;

__device__ __forceinline__ float vu_axis(float d, float L) {
  const float h = __fdiv_rn(L, 2.f);
  if (d > h) return __fsub_rn(d, L);
  if (d < -h) return __fadd_rn(d, L);
  return d;
}

__device__ __forceinline__ float len3(float x, float y, float z) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

struct BDParams {
  const float* w;
  int64_t n_pad;
  int32_t kind, axis, direction, n_bins;
  int32_t n_binned, n_from;
  int32_t binned_first, from_first;      // contiguous lists: first atom
  const int32_t* binned_idx;             // gathered lists: atom indices (else null)
  const int32_t* from_idx;
  float3 box, point;
  float position, thickness, box_max;
  int32_t* bins;                         // [frames][n_pad], -1 already
};

__global__ void __launch_bounds__(BD_THREADS) bins_distance_kernel(BDParams p) {
  __shared__ float sx[BD_TILE], sy[BD_TILE], sz[BD_TILE];
  const int t = blockIdx.y;
  const int i = blockIdx.x * BD_THREADS + threadIdx.x;
  const float* W = p.w + (int64_t)t * 3 * p.n_pad;
  const bool live = i < p.n_binned;
  const int a = live ? (p.binned_idx ? p.binned_idx[i] : p.binned_first + i) : 0;
  const float x = live ? W[a] : 0.f, y = live ? W[p.n_pad + a] : 0.f, z = live ? W[2 * p.n_pad + a] : 0.f;
  float length = 0.f;
  if (p.kind == 0) {
    // nearest member of the other list, starting from the box's largest edge
    length = p.box_max;
    for (int j0 = 0; j0 < p.n_from; j0 += BD_TILE) {
      const int nj = min(BD_TILE, p.n_from - j0);
      __syncthreads();
      for (int q = threadIdx.x; q < nj; q += BD_THREADS) {
        const int aj = p.from_idx ? p.from_idx[j0 + q] : p.from_first + j0 + q;
        sx[q] = W[aj];
        sy[q] = W[p.n_pad + aj];
        sz[q] = W[2 * p.n_pad + aj];
      }
      __syncthreads();
      if (live)
        for (int q = 0; q < nj; ++q) {
          const float tl = len3(vu_axis(__fsub_rn(x, sx[q]), p.box.x), vu_axis(__fsub_rn(y, sy[q]), p.box.y),
                                vu_axis(__fsub_rn(z, sz[q]), p.box.z));
          length = tl < length ? tl : length;
        }
    }
  } else if (p.kind == 1) {
    // dist = r - point; dist -= box * (dist / (box * 0.5)).integer()
    const float c[3] = {x, y, z}, pt[3] = {p.point.x, p.point.y, p.point.z};
    const float L[3] = {p.box.x, p.box.y, p.box.z};
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      d[k] = __fsub_rn(c[k], pt[k]);
      const float q = (float)(int)__fdiv_rn(d[k], __fmul_rn(L[k], 0.5f));
      d[k] = __fsub_rn(d[k], __fmul_rn(L[k], q));
    }
    length = len3(d[0], d[1], d[2]);
  } else {
    const float c = p.axis == 0 ? x : (p.axis == 1 ? y : z);
    const float L = p.axis == 0 ? p.box.x : (p.axis == 1 ? p.box.y : p.box.z);
    const float dist = __fsub_rn(c, p.position);
    if (p.direction == 0)  // average: |L * int(dist / (L * .5)) - dist|, the quotient in double
      length = fabsf(__fsub_rn(__fmul_rn(L, (float)(int)__ddiv_rn((double)dist, __dmul_rn((double)L, 0.5))), dist));
    else if (p.direction == 1)  // above
      length = dist < 0.f ? __fadd_rn(L, dist) : dist;
    else  // below
      length = dist < 0.f ? fabsf(dist) : __fsub_rn(L, dist);
  }
  if (!live) return;
  const int b = (int)__fdiv_rn(length, p.thickness);
  if (b >= 0 && b < p.n_bins) p.bins[(int64_t)t * p.n_pad + a] = b;
}

__global__ void bins_assign_kernel(const float* __restrict__ w, int64_t n_pad, int32_t n_atoms,
                                   int64_t n_terms, int3 nb, float3 lo, float3 hi,
                                   int32_t* __restrict__ bins) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_terms;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = i / n_atoms, a = i - t * n_atoms;
    const float* c = w + t * 3 * n_pad + a;
    const float x = c[0], y = c[n_pad], z = c[2 * n_pad];
    int32_t b = -1;
    if (x < hi.x && x > lo.x && y < hi.y && y > lo.y && z < hi.z && z > lo.z)
      b = (bin_axis(x, lo.x, hi.x, nb.x) * nb.y + bin_axis(y, lo.y, hi.y, nb.y)) * nb.z +
          bin_axis(z, lo.z, hi.z, nb.z);
    bins[t * n_pad + a] = b;
  }
}

__global__ void bins_count_kernel(const int32_t* __restrict__ bins, int64_t n_pad, int32_t n_atoms,
                                  int64_t n_terms, int32_t n_bins, unsigned long long* __restrict__ counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_terms;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = i / n_atoms, a = i - t * n_atoms;
    const int32_t b = bins[t * n_pad + a];
    if (b >= 0 && b < n_bins) atomicAdd(counts + t * n_bins + b, 1ull);
  }
}

// --- the binned displacement pass ----------------------------------------------
struct BnItem {
  int32_t pair, a0, a1, gap;
};

struct BnParams {
  const float* u;
  int64_t n_pad;
  int32_t list_first;
  const int32_t* list_idx;  // nullptr: members are list_first + i
  const int32_t* t0;
  const int32_t* t1;
  const BnItem* items;
  int32_t n_items;
  int32_t* counter;
  const int32_t* bins;  // [frames][n_pad]
  int32_t n_bins;
  int32_t persistent;
  int32_t n_fs;
  const int4* kv;
  const int32_t* kv_off;
  const float* inv_count;
  float period;
  int32_t n_gaps;
  int32_t want_d4;  // |dr|^4 column present
  int32_t stride;   // 1 + want_d4 + n_fs: |dr|^2, [|dr|^4], shells
  double* acc;     // [bin][gap][stride]
  unsigned long long* cnt;  // [bin][gap]
  int32_t staged;  // per-block shared accumulators
  int32_t n_kv_smem;    // F_s vectors staged in shared memory (0: read from kv)
  int32_t kv_smem_off;  // their byte offset in dynamic shared memory (16-byte aligned)
};

// FS: F_s shells in the columns after |dr|^2 (and |dr|^4); AXES: the columns are
// instead dx, dy, dz, dx^2, dy^2, dz^2 (msd_2d and mean_displacement per bin)
template <bool FS, bool AXES = false>
__global__ void __launch_bounds__(BN_THREADS) disp_bins_kernel(BnParams p) {
  extern __shared__ double bn_smem[];  // staged: [n_bins][stride] sums, then [n_bins] counts
  __shared__ int s_item;
  __shared__ float s_val[BN_THREADS / 32][32][2 + BN_MAX_FS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int stride = p.stride;
  double* sacc = bn_smem;
  unsigned int* scnt = reinterpret_cast<unsigned int*>(bn_smem + (size_t)p.n_bins * stride);
  int4* skv = reinterpret_cast<int4*>(reinterpret_cast<unsigned char*>(bn_smem) + p.kv_smem_off);
  if (FS)  // ordered before the first read by the loop's first barrier
    for (int i = tid; i < p.n_kv_smem; i += BN_THREADS) skv[i] = __ldg(p.kv + i);

  for (;;) {
    if (tid == 0) s_item = atomicAdd(p.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= p.n_items) break;
    const BnItem it = p.items[item];
    const int t0 = __ldg(p.t0 + it.pair), t1 = __ldg(p.t1 + it.pair);
    const float* X0 = p.u + (int64_t)t0 * 3 * p.n_pad;
    const float* X1 = p.u + (int64_t)t1 * 3 * p.n_pad;
    const int32_t* B0 = p.bins + (int64_t)t0 * p.n_pad;
    const int32_t* B1 = p.bins + (int64_t)t1 * p.n_pad;
    if (p.staged) {
      for (int i = tid; i < p.n_bins * stride; i += BN_THREADS) sacc[i] = 0.0;
      for (int i = tid; i < p.n_bins; i += BN_THREADS) scnt[i] = 0u;
      __syncthreads();
    }
    // with F_s a thread takes atoms base + tid and base + BN_THREADS + tid per
    // step: both atoms' shell sums share each vector load, and the two are
    // aggregated one after the other (the order of one atom per step)
    constexpr int H = FS ? 2 : 1;
    for (int base = it.a0; base < it.a1; base += H * BN_THREADS) {
      int bins_h[H];
      float v[H][2 + BN_MAX_FS];
      float dr[H][3];
#pragma unroll
      for (int h = 0; h < H; ++h) {
        bins_h[h] = -1;
#pragma unroll
        for (int k = 0; k < 2 + BN_MAX_FS; ++k) v[h][k] = 0.f;
        dr[h][0] = dr[h][1] = dr[h][2] = 0.f;
        const int a = base + h * BN_THREADS + tid;
        if (a < it.a1) {
          const int atom = p.list_idx ? __ldg(p.list_idx + a) : p.list_first + a;
          int b = __ldg(B0 + atom);
          if (b >= 0 && p.persistent && __ldg(B1 + atom) != b) b = -1;
          if (b >= 0) {
            const float dx = __fsub_rn(__ldg(X1 + atom), __ldg(X0 + atom));
            const float dy = __fsub_rn(__ldg(X1 + p.n_pad + atom), __ldg(X0 + p.n_pad + atom));
            const float dz = __fsub_rn(__ldg(X1 + 2 * p.n_pad + atom), __ldg(X0 + 2 * p.n_pad + atom));
            if (AXES) {
              v[h][0] = dx, v[h][1] = dy, v[h][2] = dz;
              v[h][3] = __fmul_rn(dx, dx), v[h][4] = __fmul_rn(dy, dy), v[h][5] = __fmul_rn(dz, dz);
            } else {
              v[h][0] = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
              v[h][1] = v[h][0] * v[h][0];
            }
            dr[h][0] = dx, dr[h][1] = dy, dr[h][2] = dz;
          }
          bins_h[h] = b;
        }
      }
      if (FS && (bins_h[0] >= 0 || bins_h[H - 1] >= 0)) {
        int32_t f[H][3];
#pragma unroll
        for (int h = 0; h < H; ++h)
#pragma unroll
          for (int ax = 0; ax < 3; ++ax) f[h][ax] = turns_fixed(dr[h][ax], p.period);
#pragma unroll
        for (int s = 0; s < BN_MAX_FS; ++s) {
          if (s >= p.n_fs) break;
          KSum acc_a, acc_b;
          if (p.n_kv_smem)
            list_shell_sum2<true>(skv, f[0][0], f[0][1], f[0][2], f[H - 1][0], f[H - 1][1], f[H - 1][2],
                                  p.kv_off[s], p.kv_off[s + 1], acc_a, acc_b);
          else
            list_shell_sum2<false>(p.kv, f[0][0], f[0][1], f[0][2], f[H - 1][0], f[H - 1][1], f[H - 1][2],
                                   p.kv_off[s], p.kv_off[s + 1], acc_a, acc_b);
          v[0][2 + s] = __fmul_rn(__fsub_rn(acc_a.s, acc_a.c), p.inv_count[s]);
          v[H - 1][2 + s] = __fmul_rn(__fsub_rn(acc_b.s, acc_b.c), p.inv_count[s]);
        }
      }
#pragma unroll
      for (int h = 0; h < H; ++h) {
        const int b = bins_h[h];
        // lanes of one bin: the lowest adds their terms (lane order, FP64)
        // staged columns: |dr|^2, then |dr|^4 only when asked for, then the shells
#pragma unroll
        for (int k = 0; k < 2 + BN_MAX_FS; ++k)
          if (k < stride)
            s_val[warp][lane][k] = (AXES || k == 0 || p.want_d4) ? v[h][k] : v[h][k + 1 < 2 + BN_MAX_FS ? k + 1 : k];
        __syncwarp();
        const unsigned peers = __match_any_sync(0xffffffffu, b);
        if (b >= 0 && lane == __ffs(peers) - 1) {
          const unsigned n_peers = (unsigned)__popc(peers);
          for (int k = 0; k < stride; ++k) {
            double sum = 0.0;
            for (unsigned m = peers; m; m &= m - 1) sum += (double)s_val[warp][__ffs(m) - 1][k];
            if (p.staged)
              atomicAdd(sacc + b * stride + k, sum);
            else
              atomicAdd(p.acc + ((int64_t)b * p.n_gaps + it.gap) * stride + k, sum);
          }
          if (p.staged)
            atomicAdd(scnt + b, n_peers);
          else
            atomicAdd(p.cnt + (int64_t)b * p.n_gaps + it.gap, (unsigned long long)n_peers);
        }
        __syncwarp();
      }
    }
    if (p.staged) {
      __syncthreads();
      for (int i = tid; i < p.n_bins; i += BN_THREADS) {
        if (!scnt[i]) continue;
        atomicAdd(p.cnt + (int64_t)i * p.n_gaps + it.gap, (unsigned long long)scnt[i]);
        for (int k = 0; k < stride; ++k)
          atomicAdd(p.acc + ((int64_t)i * p.n_gaps + it.gap) * stride + k, sacc[i * stride + k]);
      }
    }
    __syncthreads();
  }
}

// Compensated FP32 shared-memory accumulation: the atomic's old value gives the
// exact rounding error of the add (Knuth's TwoSum), which goes to a second
// accumulator, so hi + lo keeps the terms' sum to second order.
__device__ __forceinline__ void cadd_shared(float* hi, float* lo, float v) {
  const float old = atomicAdd(hi, v);
  const float s = __fadd_rn(old, v);
  const float bv = __fsub_rn(s, old);
  const float err = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bv)), __fsub_rn(v, bv));
  atomicAdd(lo, err);
}

// The binned pass without F_s (moments, or AXES: dx, dy, dz, dx^2, dy^2, dz^2):
// each warp adds its atoms' terms to its own compensated FP32 accumulators in
// shared memory ([warp][bin][column] hi and lo, [warp][bin] counts), and each
// item ends with one FP64 sum over the warps (warp order) per (bin, column),
// added to the (bin, gap) outputs.  Contiguous lists read four atoms per
// 16-byte load of the positions and of the bin map (rows are 128-atom aligned).
template <bool AXES>
__global__ void __launch_bounds__(BN_THREADS) disp_bins_sum_kernel(BnParams p) {
  extern __shared__ float bw_smem[];
  __shared__ int s_item[2];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int stride = AXES ? 6 : p.stride;
  const int per_warp = p.n_bins * stride;
  float* hi = bw_smem;
  float* lo = hi + BN_WARPS * per_warp;
  unsigned int* cnt = reinterpret_cast<unsigned int*>(lo + BN_WARPS * per_warp);
  for (int i = tid; i < BN_WARPS * per_warp; i += BN_THREADS) hi[i] = lo[i] = 0.f;
  for (int i = tid; i < BN_WARPS * p.n_bins; i += BN_THREADS) cnt[i] = 0u;
  float* wh = hi + warp * per_warp;
  float* wl = lo + warp * per_warp;
  unsigned int* wc = cnt + warp * p.n_bins;
  auto add = [&](int b, float dx, float dy, float dz) {
    if (b < 0) return;
    float* h = wh + b * stride;
    float* l = wl + b * stride;
    if (AXES) {
      cadd_shared(h, l, dx);
      cadd_shared(h + 1, l + 1, dy);
      cadd_shared(h + 2, l + 2, dz);
      cadd_shared(h + 3, l + 3, __fmul_rn(dx, dx));
      cadd_shared(h + 4, l + 4, __fmul_rn(dy, dy));
      cadd_shared(h + 5, l + 5, __fmul_rn(dz, dz));
    } else {
      const float d2 = sq3(dx, dy, dz);
      cadd_shared(h, l, d2);
      if (stride > 1) cadd_shared(h + 1, l + 1, d2 * d2);
    }
    atomicAdd(wc + b, 1u);
  };

  // the next item's counter slot is fetched while the current one runs
  if (tid == 0) s_item[0] = atomicAdd(p.counter, 1);
  __syncthreads();
  for (int iter = 0;; ++iter) {
    const int slot = s_item[iter & 1];
    if (slot >= p.n_items) break;
    if (tid == 0) s_item[(iter + 1) & 1] = atomicAdd(p.counter, 1);
    const BnItem it = p.items[slot];
    const int t0 = __ldg(p.t0 + it.pair), t1 = __ldg(p.t1 + it.pair);
    const float* X0 = p.u + (int64_t)t0 * 3 * p.n_pad;
    const float* X1 = p.u + (int64_t)t1 * 3 * p.n_pad;
    const int32_t* B0 = p.bins + (int64_t)t0 * p.n_pad;
    const int32_t* B1 = p.bins + (int64_t)t1 * p.n_pad;
    auto one = [&](int atom) {
      int b = __ldg(B0 + atom);
      if (b >= 0 && p.persistent && __ldg(B1 + atom) != b) b = -1;
      if (b < 0) return;
      add(b, __fsub_rn(__ldg(X1 + atom), __ldg(X0 + atom)),
          __fsub_rn(__ldg(X1 + p.n_pad + atom), __ldg(X0 + p.n_pad + atom)),
          __fsub_rn(__ldg(X1 + 2 * p.n_pad + atom), __ldg(X0 + 2 * p.n_pad + atom)));
    };
    const int lo_a = p.list_first + it.a0, hi_a = p.list_first + it.a1;
    if (!p.list_idx && (hi_a >> 2) > ((lo_a + 3) >> 2)) {
      const int v0 = (lo_a + 3) >> 2, v1 = hi_a >> 2;  // whole quads [v0, v1)
      const int64_t qp = p.n_pad >> 2;
      const float4* A0 = reinterpret_cast<const float4*>(X0);
      const float4* A1 = reinterpret_cast<const float4*>(X1);
      for (int v = v0 + tid; v < v1; v += BN_THREADS) {
        int4 b0 = __ldg(reinterpret_cast<const int4*>(B0) + v);
        if (p.persistent) {
          const int4 b1 = __ldg(reinterpret_cast<const int4*>(B1) + v);
          b0.x = b1.x == b0.x ? b0.x : -1;
          b0.y = b1.y == b0.y ? b0.y : -1;
          b0.z = b1.z == b0.z ? b0.z : -1;
          b0.w = b1.w == b0.w ? b0.w : -1;
        }
        if (b0.x < 0 && b0.y < 0 && b0.z < 0 && b0.w < 0) continue;  // no member of a bin
        const float4 x0 = __ldg(A0 + v), x1 = __ldg(A1 + v);
        const float4 y0 = __ldg(A0 + qp + v), y1 = __ldg(A1 + qp + v);
        const float4 z0 = __ldg(A0 + 2 * qp + v), z1 = __ldg(A1 + 2 * qp + v);
        add(b0.x, __fsub_rn(x1.x, x0.x), __fsub_rn(y1.x, y0.x), __fsub_rn(z1.x, z0.x));
        add(b0.y, __fsub_rn(x1.y, x0.y), __fsub_rn(y1.y, y0.y), __fsub_rn(z1.y, z0.y));
        add(b0.z, __fsub_rn(x1.z, x0.z), __fsub_rn(y1.z, y0.z), __fsub_rn(z1.z, z0.z));
        add(b0.w, __fsub_rn(x1.w, x0.w), __fsub_rn(y1.w, y0.w), __fsub_rn(z1.w, z0.w));
      }
      const int n_head = 4 * v0 - lo_a, n_tail = hi_a - 4 * v1;
      if (tid < n_head + n_tail) one(tid < n_head ? lo_a + tid : 4 * v1 + (tid - n_head));
    } else {
      for (int a = it.a0 + tid; a < it.a1; a += BN_THREADS)
        one(p.list_idx ? __ldg(p.list_idx + a) : p.list_first + a);
    }
    __syncthreads();
    // flush in FP64, warps in order; the accumulators are cleared for the next item
    for (int e = tid; e < per_warp; e += BN_THREADS) {
      double sum = 0.0;
      for (int w = 0; w < BN_WARPS; ++w) {
        sum += (double)hi[w * per_warp + e] + (double)lo[w * per_warp + e];
        hi[w * per_warp + e] = 0.f;
        lo[w * per_warp + e] = 0.f;
      }
      const int b = e / stride, k = e - b * stride;
      if (sum != 0.0) atomicAdd(p.acc + ((int64_t)b * p.n_gaps + it.gap) * stride + k, sum);
    }
    for (int b = tid; b < p.n_bins; b += BN_THREADS) {
      unsigned long long c = 0;
      for (int w = 0; w < BN_WARPS; ++w) {
        c += cnt[w * p.n_bins + b];
        cnt[w * p.n_bins + b] = 0u;
      }
      if (c) atomicAdd(p.cnt + (int64_t)b * p.n_gaps + it.gap, c);
    }
    __syncthreads();
  }
}

// --- fast particles -------------------------------------------------------------
// Fast_Particles::listkernel (src/fast_particles.cpp): over the pairs of one gap,
// a list member whose u2 = float(pow(|dr|, 2)) exceeds the threshold is fast in
// the exponential block of its start frame, int(float(t0 - frt) / float(K))
// (|dr| = sqrtf((dx*dx + dy*dy) + dz*dz), the reference's FP32 chain).
__global__ void fast_mark_kernel(const float* __restrict__ u, int64_t n_pad, int32_t list_n, int32_t list_first,
                                 const int32_t* __restrict__ list_idx, const int32_t* __restrict__ t0,
                                 const int32_t* __restrict__ t1, int32_t p0, int32_t n_pairs, int32_t frt,
                                 int32_t K, int32_t n_blocks, float min_u2, unsigned char* __restrict__ fast) {
  const int64_t n = (int64_t)n_pairs * list_n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int p = p0 + (int)(i / list_n), m = (int)(i % list_n);
    const int atom = list_idx ? list_idx[m] : list_first + m;
    const int a = t0[p], b = t1[p];
    const float* X0 = u + (int64_t)a * 3 * n_pad;
    const float* X1 = u + (int64_t)b * 3 * n_pad;
    const float dx = __fsub_rn(X1[atom], X0[atom]);
    const float dy = __fsub_rn(X1[n_pad + atom], X0[n_pad + atom]);
    const float dz = __fsub_rn(X1[2 * n_pad + atom], X0[2 * n_pad + atom]);
    const float d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    const float u2 = __double2float_rn((double)d * (double)d);
    const int blk = (int)__fdiv_rn(__fsub_rn((float)a, (float)frt), (float)K);
    if (u2 > min_u2 && blk >= 0 && blk < n_blocks) fast[(int64_t)blk * n_pad + atom] = 1;
  }
}

// membership map of the block list: frame t belongs to block int(float(t - frt) / float(K))
__global__ void fast_map_kernel(const unsigned char* __restrict__ fast, int64_t n_pad, int32_t n_atoms,
                                int64_t n_terms, int32_t frt, int32_t K, int32_t n_blocks,
                                int32_t* __restrict__ bins) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_terms;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = i / n_atoms, a = i - t * n_atoms;
    const int blk = (int)__fdiv_rn((float)(t - frt), (float)K);
    bins[t * n_pad + a] = (blk >= 0 && blk < n_blocks && fast[(int64_t)blk * n_pad + a]) ? 0 : -1;
  }
}

// members of each frame (CSR) -> one-bin map: bins[t][atom] = 0 for members
__global__ void timelist_map_kernel(const int32_t* __restrict__ offsets, const int32_t* __restrict__ idx,
                                    int32_t n_frames, int64_t n_pad, int32_t* __restrict__ bins) {
  const int t = blockIdx.y;
  if (t >= n_frames) return;
  for (int32_t e = offsets[t] + blockIdx.x * blockDim.x + threadIdx.x; e < offsets[t + 1];
       e += gridDim.x * blockDim.x)
    bins[(int64_t)t * n_pad + idx[e]] = 0;
}

static BinMap& bin_map(amdat_ctx* ctx, int32_t handle) {
  auto it = ctx->bin_maps.find(handle);
  if (it == ctx->bin_maps.end()) throw Error(AMDAT_ERR_ARGUMENT, "unknown bin map handle");
  BinMap& m = *it->second;
  if (m.n_frames != ctx->n_frames || m.n_pad != ctx->n_pad)
    throw Error(AMDAT_ERR_STATE, "the bin map was made for another trajectory");
  return m;
}

static unsigned grid_for(amdat_ctx* ctx, int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->n_sm * 16));
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_boxify(amdat_ctx* ctx, const float* lo, const float* hi) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(lo && hi, "null bounds");
    for (int d = 0; d < 3; ++d) AMDAT_REQUIRE(hi[d] > lo[d], "box bounds must satisfy hi > lo");
    const int64_t n = (int64_t)ctx->n_frames * ctx->n_atoms;
    if (n == 0) return;
    boxify_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(ctx->w.ptr, ctx->n_pad, ctx->n_atoms, n,
                                                              make_float3(lo[0], lo[1], lo[2]),
                                                              make_float3(hi[0], hi[1], hi[2]));
    check_launch("boxify_kernel");
    count_launch(ctx);
    // the FP64 copies are promoted again from the boxified planes when next needed
    ctx->u64.release();
    ctx->w64.release();
  });
}

amdat_status amdat_bins_create(amdat_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, const float* lo,
                               const float* hi, int32_t* handle) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(lo && hi && handle, "null argument");
    AMDAT_REQUIRE(nx > 0 && ny > 0 && nz > 0, "bin counts must be positive");
    AMDAT_REQUIRE((int64_t)nx * ny * nz <= (1 << 24), "at most 2^24 bins");
    auto* m = new BinMap();
    try {
      m->nx = nx, m->ny = ny, m->nz = nz;
      m->n_frames = ctx->n_frames, m->n_pad = ctx->n_pad;
      m->bin.reserve((size_t)ctx->n_frames * ctx->n_pad);
      AMDAT_CUDA(cudaMemsetAsync(m->bin.ptr, 0xff, (size_t)ctx->n_frames * ctx->n_pad * 4, ctx->stream));
      const int64_t n = (int64_t)ctx->n_frames * ctx->n_atoms;
      if (n > 0) {
        bins_assign_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(
            ctx->w.ptr, ctx->n_pad, ctx->n_atoms, n, make_int3(nx, ny, nz), make_float3(lo[0], lo[1], lo[2]),
            make_float3(hi[0], hi[1], hi[2]), m->bin.ptr);
        check_launch("bins_assign_kernel");
        count_launch(ctx);
      }
    } catch (...) {
      delete m;
      throw;
    }
    const int32_t h = ctx->next_bins++;
    ctx->bin_maps[h] = m;
    *handle = h;
  });
}

amdat_status amdat_bins_distance(amdat_ctx* ctx, int32_t kind, int32_t binned, int32_t from,
                                 const float* point, int32_t axis, int32_t direction, float position,
                                 float thickness, int32_t n_bins, int32_t* handle) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(handle != nullptr, "null handle");
    AMDAT_REQUIRE(kind >= 0 && kind <= 2, "kind must be 0 (trajectory), 1 (point) or 2 (plane)");
    AMDAT_REQUIRE(n_bins >= 1 && n_bins <= (1 << 24), "n_bins must be in [1, 2^24]");
    AMDAT_REQUIRE(thickness > 0.0f, "bin thickness must be positive");
    AMDAT_REQUIRE(kind != 1 || point != nullptr, "null point");
    AMDAT_REQUIRE(kind != 2 || (axis >= 0 && axis <= 2 && direction >= 0 && direction <= 2),
                  "plane axis must be 0..2 and direction 0 (average), 1 (above) or 2 (below)");
    const ListEntry& lb = list_entry(ctx, binned);
    const ListEntry* lf = kind == 0 ? &list_entry(ctx, from) : nullptr;
    auto* m = new BinMap();
    try {
      m->nx = (kind == 2 && axis == 0) ? n_bins : 1;
      m->ny = (kind == 2 && axis == 1) ? n_bins : 1;
      m->nz = (kind != 2 || axis == 2) ? n_bins : 1;
      m->n_frames = ctx->n_frames, m->n_pad = ctx->n_pad;
      m->bin.reserve((size_t)ctx->n_frames * ctx->n_pad);
      AMDAT_CUDA(cudaMemsetAsync(m->bin.ptr, 0xff, (size_t)ctx->n_frames * ctx->n_pad * 4, ctx->stream));
      if (lb.n > 0 && ctx->n_frames > 0) {
        BDParams p{};
        p.w = ctx->w.ptr;
        p.n_pad = ctx->n_pad;
        p.kind = kind, p.axis = axis, p.direction = direction, p.n_bins = n_bins;
        p.n_binned = lb.n;
        p.binned_first = lb.first;
        p.binned_idx = lb.contiguous ? nullptr : lb.idx.ptr;
        if (lf) {
          p.n_from = lf->n;
          p.from_first = lf->first;
          p.from_idx = lf->contiguous ? nullptr : lf->idx.ptr;
        }
        p.box = make_float3(ctx->box[0], ctx->box[1], ctx->box[2]);
        p.box_max = std::max(ctx->box[0], std::max(ctx->box[1], ctx->box[2]));
        p.point = point ? make_float3(point[0], point[1], point[2]) : make_float3(0.f, 0.f, 0.f);
        p.position = position;
        p.thickness = thickness;
        p.bins = m->bin.ptr;
        AMDAT_REQUIRE(ctx->n_frames <= 65535, "at most 65535 frames");
        dim3 grid((unsigned)ceil_div(lb.n, BD_THREADS), (unsigned)ctx->n_frames);
        bins_distance_kernel<<<grid, BD_THREADS, 0, ctx->stream>>>(p);
        check_launch("bins_distance_kernel");
        count_launch(ctx);
      }
    } catch (...) {
      delete m;
      throw;
    }
    const int32_t h = ctx->next_bins++;
    ctx->bin_maps[h] = m;
    *handle = h;
  });
}

amdat_status amdat_fast_particles(amdat_ctx* ctx, int32_t list, int32_t gap, float min_u2, int32_t* handle) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    if (!ctx->have_scheme) throw Error(AMDAT_ERR_STATE, "no time scheme set");
    AMDAT_REQUIRE(handle != nullptr, "null handle");
    const ListEntry& e = list_entry(ctx, list);
    const PairTable& P = pair_table(ctx, false, false);  // displacement_list(this, gap, false)
    AMDAT_REQUIRE(gap >= 0 && gap < P.n_gaps, "gap out of range");
    const int32_t K = ctx->scheme.n_exponential_steps, n_blocks = ctx->scheme.n_exponentials;
    const int32_t frt = ctx->scheme.frt;
    AMDAT_REQUIRE(K > 0 && n_blocks > 0, "the scheme has no exponential blocks");
    auto* m = new BinMap();
    try {
      m->nx = m->ny = m->nz = 1;
      m->n_frames = ctx->n_frames, m->n_pad = ctx->n_pad;
      m->bin.reserve((size_t)ctx->n_frames * ctx->n_pad);
      AMDAT_CUDA(cudaMemsetAsync(m->bin.ptr, 0xff, (size_t)ctx->n_frames * ctx->n_pad * 4, ctx->stream));
      unsigned char* fast = ctx->scratch.reserve((size_t)n_blocks * ctx->n_pad);
      AMDAT_CUDA(cudaMemsetAsync(fast, 0, (size_t)n_blocks * ctx->n_pad, ctx->stream));
      const int32_t p0 = P.gap_first[gap], np = P.gap_first[gap + 1] - p0;
      if (np > 0 && e.n > 0) {
        fast_mark_kernel<<<grid_for(ctx, (int64_t)np * e.n), 256, 0, ctx->stream>>>(
            ctx->u.ptr, ctx->n_pad, e.n, e.first, e.contiguous ? nullptr : e.idx.ptr, P.t0.ptr, P.t1.ptr, p0, np,
            frt, K, n_blocks, min_u2, fast);
        check_launch("fast_mark_kernel");
        count_launch(ctx);
      }
      const int64_t n = (int64_t)ctx->n_frames * ctx->n_atoms;
      if (n > 0) {
        fast_map_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(fast, ctx->n_pad, ctx->n_atoms, n, frt, K,
                                                                    n_blocks, m->bin.ptr);
        check_launch("fast_map_kernel");
        count_launch(ctx);
      }
      AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete m;
      throw;
    }
    const int32_t h = ctx->next_bins++;
    ctx->bin_maps[h] = m;
    *handle = h;
  });
}

amdat_status amdat_timelist_create(amdat_ctx* ctx, const int32_t* frame_offsets, const int32_t* atom_idx,
                                   int32_t* handle) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(frame_offsets && handle, "null argument");
    const int T = ctx->n_frames;
    AMDAT_REQUIRE(T <= 65535, "at most 65535 frames");
    AMDAT_REQUIRE(frame_offsets[0] == 0, "frame_offsets[0] must be 0");
    for (int t = 0; t < T; ++t) AMDAT_REQUIRE(frame_offsets[t + 1] >= frame_offsets[t], "frame offsets must ascend");
    const int64_t n = frame_offsets[T];
    AMDAT_REQUIRE(n == 0 || atom_idx, "null atom indices");
    for (int64_t e = 0; e < n; ++e)
      AMDAT_REQUIRE(atom_idx[e] >= 0 && atom_idx[e] < ctx->n_atoms, "atom index out of range");
    auto* m = new BinMap();
    try {
      m->nx = m->ny = m->nz = 1;
      m->n_frames = T, m->n_pad = ctx->n_pad;
      m->bin.reserve((size_t)T * ctx->n_pad);
      AMDAT_CUDA(cudaMemsetAsync(m->bin.ptr, 0xff, (size_t)T * ctx->n_pad * 4, ctx->stream));
      if (n > 0) {
        int32_t* d = reinterpret_cast<int32_t*>(ctx->scratch.reserve((size_t)(T + 1 + n) * 4));
        AMDAT_CUDA(cudaMemcpyAsync(d, frame_offsets, (size_t)(T + 1) * 4, cudaMemcpyHostToDevice, ctx->stream));
        AMDAT_CUDA(cudaMemcpyAsync(d + T + 1, atom_idx, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
        timelist_map_kernel<<<dim3(8, (unsigned)T), 256, 0, ctx->stream>>>(d, d + T + 1, T, ctx->n_pad, m->bin.ptr);
        check_launch("timelist_map_kernel");
        count_launch(ctx);
      }
      AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete m;
      throw;
    }
    const int32_t h = ctx->next_bins++;
    ctx->bin_maps[h] = m;
    *handle = h;
  });
}

amdat_status amdat_bins_free(amdat_ctx* ctx, int32_t handle) {
  return guarded([&] {
    check_ctx(ctx);
    auto it = ctx->bin_maps.find(handle);
    if (it == ctx->bin_maps.end()) throw Error(AMDAT_ERR_ARGUMENT, "unknown bin map handle");
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    delete it->second;
    ctx->bin_maps.erase(it);
  });
}

amdat_status amdat_bins_read(amdat_ctx* ctx, int32_t handle, int32_t out_flags, int32_t* bins,
                             int64_t* counts) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(out_flags == AMDAT_OUT_HOST || out_flags == AMDAT_OUT_DEVICE, "bad out_flags");
    BinMap& m = bin_map(ctx, handle);
    const int T = ctx->n_frames, N = ctx->n_atoms;
    const int32_t B = m.nx * m.ny * m.nz;
    const cudaMemcpyKind kind = out_flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (bins && N > 0)
      AMDAT_CUDA(cudaMemcpy2DAsync(bins, (size_t)N * 4, m.bin.ptr, (size_t)ctx->n_pad * 4, (size_t)N * 4, T, kind,
                                   ctx->stream));
    if (counts) {
      unsigned long long* d = reinterpret_cast<unsigned long long*>(ctx->scratch.reserve((size_t)T * B * 8));
      AMDAT_CUDA(cudaMemsetAsync(d, 0, (size_t)T * B * 8, ctx->stream));
      const int64_t n = (int64_t)T * N;
      if (n > 0) {
        bins_count_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(m.bin.ptr, ctx->n_pad, N, n, B, d);
        check_launch("bins_count_kernel");
        count_launch(ctx);
      }
      AMDAT_CUDA(cudaMemcpyAsync(counts, d, (size_t)T * B * 8, kind, ctx->stream));
    }
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

static amdat_status disp_bins_impl(amdat_ctx* ctx, int32_t list, int32_t bins, int32_t persistent,
                                   int32_t fullblock, int32_t n_shells, const int32_t* shell_offsets,
                                   const int32_t* kvec, float period, int32_t out_flags, double* sum_d2,
                                   double* sum_d4, int64_t* count, double* fs_sum, bool axes_mode,
                                   double* axis_sums) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    if (!ctx->have_scheme) throw Error(AMDAT_ERR_STATE, "no time scheme set");
    AMDAT_REQUIRE(out_flags == AMDAT_OUT_HOST || out_flags == AMDAT_OUT_DEVICE, "bad out_flags");
    AMDAT_REQUIRE(n_shells >= 0 && n_shells <= BN_MAX_FS, "n_shells must be in [0, 8]");
    AMDAT_REQUIRE(n_shells == 0 || (shell_offsets && kvec && period > 0.f), "shells need vectors and a period");
    BinMap& m = bin_map(ctx, bins);
    const ListEntry& e = list_entry(ctx, list);
    // Bin_Dynamics_Analysis enumerates displacement_list(this): fullblock 0
    const PairTable& P = pair_table(ctx, persistent ? false : fullblock != 0, false);
    const int G = P.n_gaps;
    const int32_t B = m.nx * m.ny * m.nz;
    const bool axes = axes_mode;
    AMDAT_REQUIRE(!axes || axis_sums != nullptr, "null axis_sums");
    AMDAT_REQUIRE(!axes || n_shells == 0, "per-axis sums take no shells");
    const int want_d4 = sum_d4 && !axes ? 1 : 0;
    const int stride = axes ? 6 : 1 + want_d4 + n_shells;
    // shells (list mode: one cosine per vector)
    std::vector<int4> kv;
    std::vector<int32_t> off(1, 0);
    std::vector<float> inv;
    for (int s = 0; s < n_shells; ++s) {
      AMDAT_REQUIRE(shell_offsets[s + 1] >= shell_offsets[s], "shell offsets must ascend");
      for (int q = shell_offsets[s]; q < shell_offsets[s + 1]; ++q)
        kv.push_back(make_int4(kvec[3 * q], kvec[3 * q + 1], kvec[3 * q + 2], 0));
      off.push_back((int32_t)kv.size());
      const int c = shell_offsets[s + 1] - shell_offsets[s];
      inv.push_back(c ? 1.0f / (float)c : 0.0f);
    }
    // without F_s, a grid of per-warp shared accumulators when they fit
    const size_t sum_smem = (size_t)BN_WARPS * B * (2 * (size_t)stride + 1) * 4;
    const bool sum_kernel = n_shells == 0 && sum_smem <= BN_SUM_SMEM_LIMIT;
    // items: (pair, member chunk), gap-major
    const int nch = (int)std::max<int64_t>(1, ceil_div(e.n, sum_kernel ? BN_SUM_CHUNK : BN_CHUNK));
    std::vector<BnItem> items;
    if (e.n > 0)
      for (int g = 0; g < G; ++g)
        for (int p = P.gap_first[g]; p < P.gap_first[g + 1]; ++p)
          for (int c = 0; c < nch; ++c)
            items.push_back(BnItem{p, (int32_t)((int64_t)e.n * c / nch), (int32_t)((int64_t)e.n * (c + 1) / nch), g});
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t o = 0;
    const size_t o_items = o; o = align(o + std::max<size_t>(items.size(), 1) * sizeof(BnItem));
    const size_t o_kv = o; o = align(o + std::max<size_t>(kv.size(), 1) * sizeof(int4));
    const size_t o_off = o; o = align(o + off.size() * 4);
    const size_t o_inv = o; o = align(o + std::max<size_t>(inv.size(), 1) * 4);
    const size_t o_ctr = o; o = align(o + 4);
    const size_t o_acc = o; o = align(o + (size_t)B * G * stride * 8);
    const size_t o_cnt = o; o = align(o + (size_t)B * G * 8);
    unsigned char* base = ctx->scratch.reserve(o);
    cudaStream_t st = ctx->stream;
    if (!items.empty())
      AMDAT_CUDA(cudaMemcpyAsync(base + o_items, items.data(), items.size() * sizeof(BnItem), cudaMemcpyHostToDevice, st));
    if (!kv.empty()) {
      AMDAT_CUDA(cudaMemcpyAsync(base + o_kv, kv.data(), kv.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
      AMDAT_CUDA(cudaMemcpyAsync(base + o_inv, inv.data(), inv.size() * 4, cudaMemcpyHostToDevice, st));
    }
    AMDAT_CUDA(cudaMemcpyAsync(base + o_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, st));
    AMDAT_CUDA(cudaMemsetAsync(base + o_ctr, 0, o - o_ctr, st));
    if (!items.empty()) {
      BnParams p{};
      p.u = ctx->u.ptr;
      p.n_pad = ctx->n_pad;
      p.list_first = e.first;
      p.list_idx = e.contiguous ? nullptr : e.idx.ptr;
      p.t0 = P.t0.ptr;
      p.t1 = P.t1.ptr;
      p.items = (const BnItem*)(base + o_items);
      p.n_items = (int32_t)items.size();
      p.counter = (int32_t*)(base + o_ctr);
      p.bins = m.bin.ptr;
      p.n_bins = B;
      p.persistent = persistent ? 1 : 0;
      p.n_fs = n_shells;
      p.kv = (const int4*)(base + o_kv);
      p.kv_off = (const int32_t*)(base + o_off);
      p.inv_count = (const float*)(base + o_inv);
      p.period = n_shells ? period : 1.0f;
      p.n_gaps = G;
      p.want_d4 = want_d4;
      p.stride = stride;
      p.acc = (double*)(base + o_acc);
      p.cnt = (unsigned long long*)(base + o_cnt);
      const size_t stage = (size_t)B * stride * 8 + (size_t)B * 4;
      p.staged = stage <= BN_STAGE_LIMIT ? 1 : 0;
      size_t shm = p.staged ? stage : 0;
      if (n_shells && kv.size() <= 2048) {  // the vectors in shared memory when they take at most 32 KB
        shm = (shm + 15) & ~(size_t)15;
        p.kv_smem_off = (int32_t)shm;
        p.n_kv_smem = (int32_t)kv.size();
        shm += kv.size() * sizeof(int4);
      }
      auto kern = axes ? disp_bins_kernel<false, true> : (n_shells ? disp_bins_kernel<true> : disp_bins_kernel<false>);
      if (sum_kernel) {
        kern = axes ? disp_bins_sum_kernel<true> : disp_bins_sum_kernel<false>;
        shm = sum_smem;
      }
      if (shm > 0) AMDAT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
      int per_sm = 1;
      AMDAT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BN_THREADS, shm));
      const int grid = (int)std::min<int64_t>((int64_t)ctx->n_sm * std::max(per_sm, 1), (int64_t)items.size());
      KernelTimer kt(ctx, "disp_bins_kernel");
      kern<<<grid, BN_THREADS, shm, st>>>(p);
      check_launch("disp_bins_kernel");
      count_launch(ctx);
    }
    const cudaMemcpyKind kind = out_flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    // [bin][gap][stride] -> sum_d2[bin][gap], sum_d4[bin][gap], fs_sum[bin][gap][shell],
    // or axis_sums[bin][gap][6]
    if (axes) AMDAT_CUDA(cudaMemcpyAsync(axis_sums, base + o_acc, (size_t)B * G * 6 * 8, kind, st));
    if (sum_d2 && !axes)
      AMDAT_CUDA(cudaMemcpy2DAsync(sum_d2, 8, base + o_acc, (size_t)stride * 8, 8, (size_t)B * G, kind, st));
    if (want_d4)
      AMDAT_CUDA(cudaMemcpy2DAsync(sum_d4, 8, base + o_acc + 8, (size_t)stride * 8, 8, (size_t)B * G, kind, st));
    if (fs_sum && n_shells)
      AMDAT_CUDA(cudaMemcpy2DAsync(fs_sum, (size_t)n_shells * 8, base + o_acc + 8 * (1 + want_d4), (size_t)stride * 8,
                                   (size_t)n_shells * 8, (size_t)B * G, kind, st));
    if (count) AMDAT_CUDA(cudaMemcpyAsync(count, base + o_cnt, (size_t)B * G * 8, kind, st));
    AMDAT_CUDA(cudaStreamSynchronize(st));
  });
}

amdat_status amdat_disp_bins_run(amdat_ctx* ctx, int32_t list, int32_t bins, int32_t persistent,
                                 int32_t fullblock, int32_t n_shells, const int32_t* shell_offsets,
                                 const int32_t* kvec, float period, int32_t out_flags, double* sum_d2,
                                 double* sum_d4, int64_t* count, double* fs_sum) {
  return disp_bins_impl(ctx, list, bins, persistent, fullblock, n_shells, shell_offsets, kvec, period,
                        out_flags, sum_d2, sum_d4, count, fs_sum, false, nullptr);
}

amdat_status amdat_disp_bins_axes_run(amdat_ctx* ctx, int32_t list, int32_t bins, int32_t persistent,
                                      int32_t out_flags, double* axis_sums, int64_t* count) {
  return disp_bins_impl(ctx, list, bins, persistent, 0, 0, nullptr, nullptr, 1.0f, out_flags, nullptr, nullptr,
                        count, nullptr, true, axis_sums);
}

}  // extern "C"
