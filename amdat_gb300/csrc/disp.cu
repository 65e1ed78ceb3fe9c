// Displacement family on the GPU: the per-atom kernels of
//   Mean_Square_Displacement::listkernel   (src/mean_square_displacement.cpp:164)
//   Non_Gaussian_Parameter::listkernel     (src/non_gaussian_parameter.cpp:125)
//   Incoherent_Scattering_Function::listkernel (src/incoherent_scattering_function.cpp:272)
//   Van_Hove_Self::listkernel + bin        (src/van_hove_self.cpp:98,
//                                           src/space_time_correlation_function.cpp:216)
// fused into one pass over every (list, time pair, atom) of the time-pair
// scheduler (System::displacement_list, src/system.cpp:4090).
//
// Work is cut into items (list, time pair, range of <= CHUNK list members).
// A persistent grid (a few blocks per SM) pulls items from an atomic counter.
// Per item a block streams u(t0), u(t1) for its atoms from the FP32 planes,
// accumulates |dr|^2, |dr|^4 and the F_s shell means with Kahan-compensated
// FP32 per thread, reduces them with compensated warp shuffles, and writes
// one FP64 partial per output; G_s counts go to a shared-memory histogram and
// are flushed with integer atomics (order-independent, exact).  A finalize
// kernel adds the partials of each (list, gap) in a fixed order in FP64, so
// results are deterministic run to run.
//
// F_s phases: the displacement is turned into a fixed-point fraction of the
// box per axis (units of 2^-31 turns, int32), so the phase of n.dr/L for any
// integer lattice vector n is an exact integer combination (wrapping int32
// arithmetic is arithmetic modulo whole turns) and only the final conversion
// rounds; cos is then cospif of that phase.  Two shell modes:
//   list mode    - any vector set (e.g. the reference's q-vector files):
//                  one cospif per vector;
//   octant mode  - shells closed under sign flips of each component (whole
//                  lattice shells): sum_k cos(k.dr) = sum over octant
//                  representatives of w * cos(2pi nx tx) cos(2pi ny ty)
//                  cos(2pi nz tz), with per-axis cosine tables in shared memory,
//                  so a vector costs ~0.6 FMA instead of a cosine.
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <cmath>
#include <cstring>

#include "disp_common.cuh"
#include "engine.h"
#include "umma.cuh"

namespace amdat {

constexpr int DISP_CHUNK = 4096;  // list members per item
constexpr int MAX_FS = 8;         // shells per pass
constexpr int DISP_THREADS = 256;
constexpr int FS_THREADS = 128;
constexpr int MAX_PAIRS_PER_ITEM = 64;
constexpr size_t DISP_CACHE_PLANS = 8;  // one-shot requests kept prepared

struct DispItem {
  int32_t list;  // slot in the launch's list table
  int32_t pair;  // first pair; n_pairs consecutive pairs of one gap
  int32_t a0, a1;  // member range [a0, a1) of the list
  int32_t n_pairs;
};

struct ListDev {
  int32_t n;
  int32_t first;
  const int32_t* idx;  // nullptr: members are atoms first..first+n-1
};

// One item as the kernel reads it, stored in processing order: everything a
// block needs to start streaming in one 48-byte record, so a single read (not
// a chain of dependent table reads) precedes an item's loads.
struct alignas(16) DispDesc {
  int32_t item;    // row of the item's partials
  int32_t unit;    // work-unit slot (G_s output row)
  int32_t a0, a1;  // member range [a0, a1)
  int32_t t0, t1, gap;
  int32_t first;        // members are first + a when idx is null
  const int32_t* idx;   // member atom indexes, or null
  int32_t n_pairs;      // > 1: pairs (frames[pf + i].x, .y), i < n_pairs, all of this gap
  int32_t pf;
};
static_assert(sizeof(DispDesc) == 48, "descriptor layout");

struct DispParams {
  const float* u;
  int64_t n_pad;
  const DispDesc* desc;  // [n_items], processing order
  const int2* frames;    // (t0, t1) of the pairs of multi-pair items
  int32_t n_items;
  int32_t* counter;
  double* part;  // [n_items][n_out]
  int32_t n_out;
  int32_t want_moments;
  // G_s
  unsigned long long* gs;  // [list][gap][bin]
  int32_t n_gaps;
  int32_t n_bins;
  float bin_size;
  // F_s
  int32_t n_fs;              // shells in this pass (<= MAX_FS)
  int32_t fs_mode;           // 0 none, 1 list, 2 octant
  const int4* kv;            // list mode: (nx, ny, nz, _) per vector
  const int32_t* kv_off;     // [n_fs + 1]
  const float* inv_count;    // [n_fs] 1 / vectors in shell
  int32_t nmax;              // octant mode table size - 1
  float period;              // L of k = 2 pi n / L
  int32_t n_rep_smem;        // F_s vectors (list) or representatives (octant) of the pass in shared memory (0: read from kv)
};

// octant mode: the compensated sum over one shell's representatives (blocks of
// 32 terms, each block added to the sum), reading the representatives from
// shared memory or through the read-only cache
template <bool SMEM>
__device__ __forceinline__ KSum octant_shell_sum(const int4* R, const float* T, int v_begin, int v_end) {
  KSum acc = {0.f, 0.f};
  for (int v0 = v_begin; v0 < v_end; v0 += 32) {
    const int v1 = min(v0 + 32, v_end);
    float blk = 0.f;
#pragma unroll 4
    for (int v = v0; v < v1; ++v) {
      const int4 r = SMEM ? R[v] : __ldg(R + v);
      blk = fmaf(__int_as_float(r.w) * T[r.x] * T[r.y], T[r.z], blk);
    }
    kadd(acc, blk);
  }
  if ((v_end - v_begin) % 32 == 0) kadd(acc, 0.f);  // the closing (empty) block
  return acc;
}

template <int MODE, bool GS>
__global__ void __launch_bounds__(MODE == 0 ? DISP_THREADS : FS_THREADS)
    disp_mixed_kernel(DispParams p) {
  extern __shared__ float smem[];
  __shared__ int s_item[2];  // counter slots of the item being processed and the next one
  __shared__ KSum s_red[(MODE == 0 ? DISP_THREADS : FS_THREADS) / 32][2 + MAX_FS];
  unsigned int* hist = reinterpret_cast<unsigned int*>(smem);  // [n_bins] when GS
  float* tab = smem + (GS ? ((p.n_bins + 3) & ~3) : 0);         // octant tables
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
  const int n_fs = MODE ? p.n_fs : 0;
  // F_s: the pass's vectors (list mode) or representatives (octant mode, after
  // the tables) in shared memory, when they fit
  int4* reps = reinterpret_cast<int4*>(tab + (MODE == 2 ? 3 * (p.nmax + 1) * nthr : 0));
  if (MODE != 0 && p.n_rep_smem)
    for (int i = tid; i < p.n_rep_smem; i += nthr) reps[i] = __ldg(p.kv + p.kv_off[0] + i);

  // the next item's counter slot is fetched while the current item is
  // processed (two slots: slot i & 1 is read after the barrier that ends item
  // i - 1 and written again only after the barriers inside item i + 1); the
  // item itself is one descriptor read
  if (tid == 0) s_item[0] = atomicAdd(p.counter, 1);
  __syncthreads();
  for (int iter = 0;; ++iter) {
    const int slot = s_item[iter & 1];
    if (slot >= p.n_items) break;
    if (tid == 0) s_item[(iter + 1) & 1] = atomicAdd(p.counter, 1);
    const DispDesc it = p.desc[slot];
    const int item = it.item, g = it.gap;
    const ListDev L{0, it.first, it.idx};
    const float* X0 = p.u + (int64_t)it.t0 * 3 * p.n_pad;
    const float* X1 = p.u + (int64_t)it.t1 * 3 * p.n_pad;
    if (GS)
      for (int b = tid; b < p.n_bins; b += nthr) hist[b] = 0u;
    if (GS) __syncthreads();

    KSum m2 = {0.f, 0.f}, m4 = {0.f, 0.f};
    KSum fs[MAX_FS];
#pragma unroll
    for (int s = 0; s < MAX_FS; ++s) fs[s] = KSum{0.f, 0.f};

    int a_start = it.a0 + tid;
    if (MODE == 0 && !GS && it.n_pairs > 1) {
      // a small member range over several pairs of one gap: the block walks
      // the flat (pair, member) range, element e = pair * nm + member, so
      // every thread has loads in flight even when nm is below the block size
      const int nm = it.a1 - it.a0, total = it.n_pairs * nm;
      const int q = nthr / nm, r = nthr - q * nm;  // a stride of nthr elements
      int pr = tid / nm, a = tid - pr * nm;
      const int2* F = p.frames + it.pf;
      auto offsets = [&](int64_t& o0, int64_t& o1) {
        const int2 tt = __ldg(F + pr);
        const int atom = L.idx ? __ldg(L.idx + it.a0 + a) : L.first + it.a0 + a;
        o0 = (int64_t)tt.x * 3 * p.n_pad + atom;
        o1 = (int64_t)tt.y * 3 * p.n_pad + atom;
        pr += q;
        a += r;
        if (a >= nm) {
          a -= nm;
          ++pr;
        }
      };
      int e = tid;
      constexpr int MP_BATCH = 4;
      for (; e + (MP_BATCH - 1) * nthr < total; e += MP_BATCH * nthr) {
        int64_t o0[MP_BATCH], o1[MP_BATCH];
#pragma unroll
        for (int k = 0; k < MP_BATCH; ++k) offsets(o0[k], o1[k]);
        float d[MP_BATCH][3];
#pragma unroll
        for (int k = 0; k < MP_BATCH; ++k)
#pragma unroll
          for (int ax = 0; ax < 3; ++ax)
            d[k][ax] = __fsub_rn(__ldg(p.u + o1[k] + ax * p.n_pad), __ldg(p.u + o0[k] + ax * p.n_pad));
#pragma unroll
        for (int k = 0; k < MP_BATCH; ++k) {
          const float d2 = fmaf(d[k][2], d[k][2], fmaf(d[k][1], d[k][1], d[k][0] * d[k][0]));
          kadd(m2, d2);
          kadd(m4, d2 * d2);
        }
      }
      for (; e < total; e += nthr) {
        int64_t o0, o1;
        offsets(o0, o1);
        const float dx = __fsub_rn(__ldg(p.u + o1), __ldg(p.u + o0));
        const float dy = __fsub_rn(__ldg(p.u + o1 + p.n_pad), __ldg(p.u + o0 + p.n_pad));
        const float dz = __fsub_rn(__ldg(p.u + o1 + 2 * p.n_pad), __ldg(p.u + o0 + 2 * p.n_pad));
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        kadd(m2, d2);
        kadd(m4, d2 * d2);
      }
      a_start = it.a1;  // nothing left for the single-pair loops
    } else if (MODE == 0 && !L.idx && (L.first + it.a1) / 4 > (L.first + it.a0 + 3) / 4) {
      // contiguous members: one 16-byte load per plane and frame brings four
      // consecutive atoms (planes start on 128-atom boundaries); the < 4 atoms
      // before the first and after the last whole quad go one per thread
      auto term = [&](float dx, float dy, float dz) {
        const float e = sq3(dx, dy, dz);
        kadd(m2, e);
        kadd(m4, e * e);
        if (GS) {
          // the reference's FP32 chain: sqrt((dx*dx + dy*dy) + dz*dz) / bin_size
          const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
          const int b = (int)__fdiv_rn(__fsqrt_rn(s2), p.bin_size);
          if (b >= 0 && b < p.n_bins) atomicAdd(hist + b, 1u);
        }
      };
      const int lo = L.first + it.a0, hi = L.first + it.a1;
      const int v0 = (lo + 3) >> 2, v1 = hi >> 2;  // whole quads [v0, v1)
      const float4* A0 = reinterpret_cast<const float4*>(X0);
      const float4* A1 = reinterpret_cast<const float4*>(X1);
      const int64_t qp = p.n_pad >> 2;  // quads per plane
      for (int v = v0 + tid; v < v1; v += nthr) {
        const float4 x0 = __ldg(A0 + v), x1 = __ldg(A1 + v);
        const float4 y0 = __ldg(A0 + qp + v), y1 = __ldg(A1 + qp + v);
        const float4 z0 = __ldg(A0 + 2 * qp + v), z1 = __ldg(A1 + 2 * qp + v);
        term(__fsub_rn(x1.x, x0.x), __fsub_rn(y1.x, y0.x), __fsub_rn(z1.x, z0.x));
        term(__fsub_rn(x1.y, x0.y), __fsub_rn(y1.y, y0.y), __fsub_rn(z1.y, z0.y));
        term(__fsub_rn(x1.z, x0.z), __fsub_rn(y1.z, y0.z), __fsub_rn(z1.z, z0.z));
        term(__fsub_rn(x1.w, x0.w), __fsub_rn(y1.w, y0.w), __fsub_rn(z1.w, z0.w));
      }
      const int n_head = 4 * v0 - lo, n_tail = hi - 4 * v1;
      if (tid < n_head + n_tail) {
        const int atom = tid < n_head ? lo + tid : 4 * v1 + (tid - n_head);
        term(__fsub_rn(__ldg(X1 + atom), __ldg(X0 + atom)),
             __fsub_rn(__ldg(X1 + p.n_pad + atom), __ldg(X0 + p.n_pad + atom)),
             __fsub_rn(__ldg(X1 + 2 * p.n_pad + atom), __ldg(X0 + 2 * p.n_pad + atom)));
      }
      a_start = it.a1;  // nothing left for the loops below
    } else if (MODE == 0 && !GS) {
      // gathered members (index lists): MSD_BATCH atoms' six loads each are
      // issued before any of them is used (the pass is load-latency bound)
      constexpr int MSD_BATCH = 4;  // 8 costs occupancy (registers) and is slower
      for (; a_start + (MSD_BATCH - 1) * nthr < it.a1; a_start += MSD_BATCH * nthr) {
        int at[MSD_BATCH];
#pragma unroll
        for (int k = 0; k < MSD_BATCH; ++k)
          at[k] = L.idx ? __ldg(L.idx + a_start + k * nthr) : L.first + a_start + k * nthr;
        float d[MSD_BATCH][3];
#pragma unroll
        for (int k = 0; k < MSD_BATCH; ++k) {
          d[k][0] = __fsub_rn(__ldg(X1 + at[k]), __ldg(X0 + at[k]));
          d[k][1] = __fsub_rn(__ldg(X1 + p.n_pad + at[k]), __ldg(X0 + p.n_pad + at[k]));
          d[k][2] = __fsub_rn(__ldg(X1 + 2 * p.n_pad + at[k]), __ldg(X0 + 2 * p.n_pad + at[k]));
        }
        if (p.want_moments) {
#pragma unroll
          for (int k = 0; k < MSD_BATCH; ++k) {
            const float d2 = fmaf(d[k][2], d[k][2], fmaf(d[k][1], d[k][1], d[k][0] * d[k][0]));
            kadd(m2, d2);
            kadd(m4, d2 * d2);
          }
        }
      }
    }
    if (MODE == 1 && !GS) {
      // list-mode F_s: a thread's atoms a and a + nthr together (the same atoms
      // and the same order of every sum as one atom per step below)
      for (; a_start + nthr < it.a1; a_start += 2 * nthr) {
        const int atom_a = L.idx ? __ldg(L.idx + a_start) : L.first + a_start;
        const int atom_b = L.idx ? __ldg(L.idx + a_start + nthr) : L.first + a_start + nthr;
        float d[2][3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          d[0][ax] = __fsub_rn(__ldg(X1 + ax * p.n_pad + atom_a), __ldg(X0 + ax * p.n_pad + atom_a));
          d[1][ax] = __fsub_rn(__ldg(X1 + ax * p.n_pad + atom_b), __ldg(X0 + ax * p.n_pad + atom_b));
        }
        if (p.want_moments) {
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const float d2 = fmaf(d[k][2], d[k][2], fmaf(d[k][1], d[k][1], d[k][0] * d[k][0]));
            kadd(m2, d2);
            kadd(m4, d2 * d2);
          }
        }
        int32_t f[2][3];
#pragma unroll
        for (int k = 0; k < 2; ++k)
#pragma unroll
          for (int ax = 0; ax < 3; ++ax) f[k][ax] = turns_fixed(d[k][ax], p.period);
        for (int s = 0; s < n_fs; ++s) {
          KSum acc_a, acc_b;
          if (p.n_rep_smem)
            list_shell_sum2<true>(reps - p.kv_off[0], f[0][0], f[0][1], f[0][2], f[1][0], f[1][1], f[1][2],
                                  p.kv_off[s], p.kv_off[s + 1], acc_a, acc_b);
          else
            list_shell_sum2<false>(p.kv, f[0][0], f[0][1], f[0][2], f[1][0], f[1][1], f[1][2], p.kv_off[s],
                                   p.kv_off[s + 1], acc_a, acc_b);
          kadd(fs[s], __fmul_rn(__fsub_rn(acc_a.s, acc_a.c), p.inv_count[s]));
          kadd(fs[s], __fmul_rn(__fsub_rn(acc_b.s, acc_b.c), p.inv_count[s]));
        }
      }
    }
    for (int a = a_start; a < it.a1; a += nthr) {
      const int atom = L.idx ? __ldg(L.idx + a) : L.first + a;
      const float dx = __fsub_rn(__ldg(X1 + atom), __ldg(X0 + atom));
      const float dy = __fsub_rn(__ldg(X1 + p.n_pad + atom), __ldg(X0 + p.n_pad + atom));
      const float dz = __fsub_rn(__ldg(X1 + 2 * p.n_pad + atom), __ldg(X0 + 2 * p.n_pad + atom));
      if (p.want_moments) {
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        kadd(m2, d2);
        kadd(m4, d2 * d2);
      }
      if (GS) {
        // the reference's FP32 chain: sqrt((dx*dx + dy*dy) + dz*dz) / bin_size
        const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        const int b = (int)__fdiv_rn(__fsqrt_rn(s2), p.bin_size);
        if (b >= 0 && b < p.n_bins) atomicAdd(hist + b, 1u);
      }
      if (MODE == 1) {
        const int32_t fx = turns_fixed(dx, p.period);
        const int32_t fy = turns_fixed(dy, p.period);
        const int32_t fz = turns_fixed(dz, p.period);
        for (int s = 0; s < n_fs; ++s) {
          const KSum acc = p.n_rep_smem
                               ? list_shell_sum<true>(reps - p.kv_off[0], fx, fy, fz, p.kv_off[s], p.kv_off[s + 1])
                               : list_shell_sum<false>(p.kv, fx, fy, fz, p.kv_off[s], p.kv_off[s + 1]);
          kadd(fs[s], __fmul_rn(__fsub_rn(acc.s, acc.c), p.inv_count[s]));
        }
      }
      if (MODE == 2) {
        // per-thread cosine tables cos(2 pi n t_axis), n = 0..nmax, layout
        // [axis][n][thread] (conflict-free: each thread owns a column)
        const int32_t f[3] = {turns_fixed(dx, p.period), turns_fixed(dy, p.period),
                              turns_fixed(dz, p.period)};
        const int stride = (p.nmax + 1) * nthr;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
          for (int n = 0; n <= p.nmax; ++n)
            tab[ax * stride + n * nthr + tid] = cos_fixed((int32_t)((uint32_t)n * (uint32_t)f[ax]));
        // octant representatives: (x, y, z) table offsets for FS_THREADS threads
        // (the launch's block size in this mode), .w = multiplicity as FP32 bits;
        // terms summed in blocks of 32, each block added to the compensated sum
        const float* T = tab + tid;
        for (int s = 0; s < n_fs; ++s) {
          const KSum acc = p.n_rep_smem
                               ? octant_shell_sum<true>(reps - p.kv_off[0], T, p.kv_off[s], p.kv_off[s + 1])
                               : octant_shell_sum<false>(p.kv, T, p.kv_off[s], p.kv_off[s + 1]);
          kadd(fs[s], __fmul_rn(__fsub_rn(acc.s, acc.c), p.inv_count[s]));
        }
      }
    }

    // block reduction of the compensated sums
    const int n_red = 2 + n_fs;
    for (int k = 0; k < n_red; ++k) {
      KSum v = k == 0 ? m2 : (k == 1 ? m4 : fs[0]);
      if (MODE) {
#pragma unroll
        for (int s = 0; s < MAX_FS; ++s)
          if (k == 2 + s) v = fs[s];
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v = kmerge(v, kshfl(v, off));
      if (lane == 0) s_red[warp][k] = v;
    }
    __syncthreads();
    if (tid < n_red) {
      double acc = 0.0;
      for (int w = 0; w < nwarp; ++w) acc += (double)s_red[w][tid].s - (double)s_red[w][tid].c;
      p.part[(int64_t)item * p.n_out + tid] = acc;
    }
    if (GS) {
      __syncthreads();
      unsigned long long* dst = p.gs + ((int64_t)it.unit * p.n_gaps + g) * p.n_bins;
      for (int b = tid; b < p.n_bins; b += nthr)
        if (hist[b]) atomicAdd(dst + b, (unsigned long long)hist[b]);
    }
    __syncthreads();
  }
}

// Sums the partials of each (unit, gap) in a fixed order (FP64): one warp per
// output (lanes stride over the items, then a fixed shuffle tree).
__global__ void disp_finalize_kernel(const double* __restrict__ part, int32_t n_out,
                                     const int32_t* __restrict__ item_first,  // [n_lg + 1]
                                     int32_t n_lg, double* __restrict__ out_d2,
                                     double* __restrict__ out_d4, double* __restrict__ out_fs,
                                     int32_t fs_stride, int32_t fs_offset, int32_t n_fs,
                                     int32_t want_moments) {
  const int n_red = 2 + n_fs, lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (gw >= (int64_t)n_lg * n_red) return;
  const int lg = (int)(gw / n_red), k = (int)(gw % n_red);
  if (k < 2 && !want_moments) return;
  const int i0 = item_first[lg], i1 = item_first[lg + 1];
  double acc = 0.0;
  for (int i = i0 + lane; i < i1; i += 32) acc += part[(int64_t)i * n_out + k];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    if (k == 0 && out_d2) out_d2[lg] = acc;
    if (k == 1 && out_d4) out_d4[lg] = acc;
    if (k >= 2 && out_fs) out_fs[(int64_t)lg * fs_stride + fs_offset + (k - 2)] = acc;
  }
}

// ---------------------------------------------------------------------------
// bulk-copy-staged MSD + NGP moments (members contiguous, no F_s, no G_s;
// selected with AMDAT_DISP_KERNEL=bulk when a plan is made).
// One producer thread walks the items (work counter shared with the other
// blocks) and streams each (pair, up to BK_SEG atoms) segment's six planes (x,
// y, z at t0 and t1) into a BK_STAGES-deep shared-memory ring with
// cp.async.bulk, running ahead across items; the consumer warps reduce each
// segment from shared memory (16-byte loads of four atoms per plane) and write
// an item's partials after its last segment.  The few atoms before the first
// and after the last whole quad of a pair's range take direct loads.
// ---------------------------------------------------------------------------
constexpr int BK_CONSUMERS = 8;   // consumer warps
constexpr int BK_THREADS = 32 * (BK_CONSUMERS + 1);
constexpr uint32_t BK_WAIT = 1u << 20;  // try_wait calls of <= 1 us

struct BkMeta {
  int32_t item;      // < 0: no more work
  int32_t s_lo, s_hi;  // whole-quad atom range in the stage
  int32_t h_lo, h_hi;  // atoms loaded directly (the pair's ragged ends)
  int32_t t_lo, t_hi;
  int32_t t0, t1;
  int32_t last;      // the item's last segment
};
// BK_SEG atoms per segment (a multiple of 4), BK_STAGES ring stages
template <int BK_SEG, int BK_STAGES>
struct BkSmem {
  float buf[BK_STAGES][6][BK_SEG];
  BkMeta meta[BK_STAGES];
  uint64_t full[BK_STAGES], empty[BK_STAGES];
  // the item reductions alternate between two buffers: consumer warps fill
  // red[b] and arrive on red_full[b]; warp 0 sums it and arrives on red_empty[b]
  KSum red[2][BK_CONSUMERS][2];
  uint64_t red_full[2], red_empty[2];
  volatile int bad;
};

template <int BK_SEG, int BK_STAGES>
__global__ void __launch_bounds__(BK_THREADS) disp_bulk_kernel(DispParams p, int* __restrict__ err) {
  extern __shared__ unsigned char bk_raw[];
  using Smem = BkSmem<BK_SEG, BK_STAGES>;
  Smem& S = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(bk_raw) + 127) & ~(uintptr_t)127);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    for (int s = 0; s < BK_STAGES; ++s) {
      umma::mbar_init(&S.full[s], 1);
      umma::mbar_init(&S.empty[s], BK_CONSUMERS);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(&S.red_full[b], BK_CONSUMERS);
      umma::mbar_init(&S.red_empty[b], 1);
    }
    umma::fence_mbarrier_init();
    S.bad = 0;
  }
  __syncthreads();
  const int64_t plane = p.n_pad;
  if (warp == BK_CONSUMERS) {
    // ---- producer
    if (lane == 0) {
      int seg = 0;
      auto next_stage = [&](int& st) -> bool {
        st = seg % BK_STAGES;
        return !S.bad && umma::mbar_wait(&S.empty[st], ((seg / BK_STAGES) & 1) ^ 1, BK_WAIT);
      };
      bool ok = true;
      for (;;) {
        const int slot = atomicAdd(p.counter, 1);
        if (slot >= p.n_items) break;
        const DispDesc d = p.desc[slot];
        const int lo = d.first + d.a0, hi = d.first + d.a1;
        // whole quads [lo4, hi4); ranges under eight atoms go by direct loads
        int lo4 = (lo + 3) & ~3, hi4 = hi & ~3;
        if (hi - lo < 8) lo4 = hi4 = lo;
        for (int pi = 0; pi < d.n_pairs && ok; ++pi) {
          const int2 tt = d.n_pairs > 1 ? __ldg(p.frames + d.pf + pi) : make_int2(d.t0, d.t1);
          int s_lo = lo4;
          do {
            const int s_hi = min(s_lo + BK_SEG, hi4);
            int st;
            if (!next_stage(st)) {
              ok = false;
              break;
            }
            const bool first = s_lo == lo4, end = s_hi == hi4;
            BkMeta& m = S.meta[st];
            m.item = d.item;
            m.s_lo = s_lo;
            m.s_hi = s_hi;
            m.h_lo = first ? lo : 0;
            m.h_hi = first ? (hi - lo < 8 ? hi : lo4) : 0;
            m.t_lo = end && hi - lo >= 8 ? hi4 : 0;
            m.t_hi = end && hi - lo >= 8 ? hi : 0;
            m.t0 = tt.x;
            m.t1 = tt.y;
            m.last = end && pi == d.n_pairs - 1;
            const uint32_t bytes = (uint32_t)(s_hi - s_lo) * 4u;
            if (bytes) {
              umma::mbar_expect_tx(&S.full[st], 6u * bytes);
#pragma unroll
              for (int k = 0; k < 6; ++k) {
                const int t = k < 3 ? tt.x : tt.y;
                umma::bulk_g2s(S.buf[st][k], p.u + ((int64_t)t * 3 + (k % 3)) * plane + s_lo, bytes, &S.full[st]);
              }
            } else {
              umma::mbar_arrive(&S.full[st]);
            }
            ++seg;
            s_lo = s_hi;
          } while (s_lo < hi4);
        }
        if (!ok) break;
      }
      // the stop marker; after a failure the consumers leave through the error flag
      bool stopped = false;
      int st;
      if (ok && next_stage(st)) {
        S.meta[st].item = -1;
        umma::mbar_arrive(&S.full[st]);
        stopped = true;
      }
      if (!stopped) S.bad = 1;
      // copies still in flight land before the block exits (segments whose
      // stage no later issue reused)
      for (int s = max(0, seg - BK_STAGES + (stopped ? 1 : 0)); s < seg; ++s)
        umma::mbar_wait(&S.full[s % BK_STAGES], (s / BK_STAGES) & 1, BK_WAIT);
    }
  } else {
    // ---- consumers
    KSum m2 = {0.f, 0.f}, m4 = {0.f, 0.f};
    const int ct = tid;  // 0 .. 32 * BK_CONSUMERS - 1
    auto term = [&](float dx, float dy, float dz) {
      const float e = sq3(dx, dy, dz);
      kadd(m2, e);
      kadd(m4, e * e);
    };
    int n_done = 0;  // items this block's consumers finished
    for (int seg = 0;; ++seg) {
      const int st = seg % BK_STAGES;
      bool ok = true;
      if (lane == 0) ok = umma::mbar_wait(&S.full[st], (seg / BK_STAGES) & 1, BK_WAIT) && !S.bad;
      if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
        S.bad = 1;
        break;
      }
      const BkMeta m = S.meta[st];
      if (m.item < 0) break;
      const int nq = (m.s_hi - m.s_lo) >> 2;
      const float4* P[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) P[k] = reinterpret_cast<const float4*>(S.buf[st][k]);
      for (int q = ct; q < nq; q += 32 * BK_CONSUMERS) {
        const float4 x0 = P[0][q], y0 = P[1][q], z0 = P[2][q], x1 = P[3][q], y1 = P[4][q], z1 = P[5][q];
        term(__fsub_rn(x1.x, x0.x), __fsub_rn(y1.x, y0.x), __fsub_rn(z1.x, z0.x));
        term(__fsub_rn(x1.y, x0.y), __fsub_rn(y1.y, y0.y), __fsub_rn(z1.y, z0.y));
        term(__fsub_rn(x1.z, x0.z), __fsub_rn(y1.z, y0.z), __fsub_rn(z1.z, z0.z));
        term(__fsub_rn(x1.w, x0.w), __fsub_rn(y1.w, y0.w), __fsub_rn(z1.w, z0.w));
      }
      const int nh = m.h_hi - m.h_lo, nt = m.t_hi - m.t_lo;
      if (ct < nh + nt) {
        const int atom = ct < nh ? m.h_lo + ct : m.t_lo + (ct - nh);
        const float* X0 = p.u + (int64_t)m.t0 * 3 * plane;
        const float* X1 = p.u + (int64_t)m.t1 * 3 * plane;
        term(__fsub_rn(__ldg(X1 + atom), __ldg(X0 + atom)),
             __fsub_rn(__ldg(X1 + plane + atom), __ldg(X0 + plane + atom)),
             __fsub_rn(__ldg(X1 + 2 * plane + atom), __ldg(X0 + 2 * plane + atom)));
      }
      __syncwarp();
      if (lane == 0) umma::mbar_arrive(&S.empty[st]);
      if (m.last) {
        // the item's partials: warp shuffles, then FP64 over the consumer warps
        // in warp order (buffer b = item parity; use u of it waits for warp 0
        // to have read use u - 1)
        const int b = n_done & 1, u = n_done >> 1;
        KSum v[2] = {m2, m4};
#pragma unroll
        for (int k = 0; k < 2; ++k)
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) v[k] = kmerge(v[k], kshfl(v[k], off));
        if (lane == 0) ok = umma::mbar_wait(&S.red_empty[b], (u & 1) ^ 1, BK_WAIT);
        if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
          S.bad = 1;
          break;
        }
        if (lane == 0) {
          S.red[b][warp][0] = v[0];
          S.red[b][warp][1] = v[1];
          umma::mbar_arrive(&S.red_full[b]);
        }
        if (warp == 0) {
          if (lane == 0) ok = umma::mbar_wait(&S.red_full[b], u & 1, BK_WAIT);
          if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
            S.bad = 1;
            break;
          }
          __syncwarp();  // lane 1 reads after lane 0's acquire
          if (lane < 2) {
            double acc = 0.0;
            for (int w = 0; w < BK_CONSUMERS; ++w)
              acc += (double)S.red[b][w][lane].s - (double)S.red[b][w][lane].c;
            p.part[(int64_t)m.item * p.n_out + lane] = acc;
          }
          __syncwarp();
          if (lane == 0) umma::mbar_arrive(&S.red_empty[b]);
        }
        ++n_done;
        m2 = KSum{0.f, 0.f};
        m4 = KSum{0.f, 0.f};
      }
    }
  }
  __syncthreads();
  if (tid == 0 && S.bad) atomicExch(err, 1);
}

// Sums each list's membership classes into the list's outputs (FP64, classes
// in ascending order per lane, then a fixed shuffle tree): one warp per
// (list, gap, column).
__global__ void disp_combine_kernel(int32_t G, int32_t S, int32_t n_lg, const int32_t* __restrict__ lu_off,
                                    const int32_t* __restrict__ lu_units, const double* __restrict__ ud2,
                                    const double* __restrict__ ud4, const double* __restrict__ ufs,
                                    double* __restrict__ d2, double* __restrict__ d4, double* __restrict__ fs) {
  const int n_red = 2 + S, S1 = S > 0 ? S : 1, lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (gw >= (int64_t)n_lg * n_red) return;
  const int lg = (int)(gw / n_red), k = (int)(gw % n_red), l = lg / G, g = lg % G;
  const int u0 = lu_off[l], u1 = lu_off[l + 1];
  double acc = 0.0;
  for (int i = u0 + lane; i < u1; i += 32) {
    const int64_t ug = (int64_t)lu_units[i] * G + g;
    acc += k == 0 ? ud2[ug] : (k == 1 ? ud4[ug] : ufs[ug * S1 + (k - 2)]);
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    if (k == 0) d2[lg] = acc;
    else if (k == 1) d4[lg] = acc;
    else fs[(int64_t)lg * S1 + (k - 2)] = acc;
  }
}

// G_s counts of each list: the sums of its classes' counts (integers)
__global__ void disp_combine_gs_kernel(int32_t G, int32_t NB, const int32_t* __restrict__ lu_off,
                                       const int32_t* __restrict__ lu_units,
                                       const unsigned long long* __restrict__ ugs,
                                       unsigned long long* __restrict__ gs) {
  const int lg = blockIdx.x, l = lg / G, g = lg % G;
  const int u0 = lu_off[l], u1 = lu_off[l + 1];
  for (int b = threadIdx.x; b < NB; b += blockDim.x) {
    unsigned long long c = 0ull;
    for (int i = u0; i < u1; ++i) c += ugs[((int64_t)lu_units[i] * G + g) * NB + b];
    gs[(int64_t)lg * NB + b] = c;
  }
}

// ---------------------------------------------------------------------------
// plain FP64 path: one thread per (pair, atom), FP64 arithmetic, direct cos,
// block reduction then one FP64 atomic per block and output
// ---------------------------------------------------------------------------
struct PlainParams {
  const double* u;
  int64_t n_pad;
  const int32_t* t0;
  const int32_t* t1;
  const int32_t* gap;
  int64_t n_pairs;
  ListDev list;
  int32_t blocks_per_pair;
  double* d2;  // [G]
  double* d4;
  double* fs;  // [G][S]
  int32_t n_shells;
  const int4* kv;
  const int32_t* kv_off;
  double two_pi_over_l;
  unsigned long long* gs;
  int32_t n_bins;
  double bin_size;
};

__global__ void disp_plain_kernel(PlainParams p) {
  const int64_t pair = blockIdx.x / p.blocks_per_pair;
  const int a = (int)(blockIdx.x % p.blocks_per_pair) * blockDim.x + threadIdx.x;
  __shared__ double red[32];
  double v2 = 0, v4 = 0;
  double dx = 0, dy = 0, dz = 0;
  bool live = a < p.list.n;
  const int g = p.gap[pair];
  if (live) {
    const int atom = p.list.idx ? p.list.idx[a] : p.list.first + a;
    const double* X0 = p.u + (int64_t)p.t0[pair] * 3 * p.n_pad;
    const double* X1 = p.u + (int64_t)p.t1[pair] * 3 * p.n_pad;
    dx = X1[atom] - X0[atom];
    dy = X1[p.n_pad + atom] - X0[p.n_pad + atom];
    dz = X1[2 * p.n_pad + atom] - X0[2 * p.n_pad + atom];
    v2 = dx * dx + dy * dy + dz * dz;
    v4 = v2 * v2;
    if (p.n_bins > 0) {
      const int b = (int)(sqrt(v2) / p.bin_size);
      if (b >= 0 && b < p.n_bins) atomicAdd(p.gs + (int64_t)g * p.n_bins + b, 1ull);
    }
  }
  auto block_sum = [&](double v) -> double {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    return t;
  };
  double s2 = block_sum(v2);
  double s4 = block_sum(v4);
  if (threadIdx.x == 0) {
    atomicAdd(p.d2 + g, s2);
    atomicAdd(p.d4 + g, s4);
  }
  for (int s = 0; s < p.n_shells; ++s) {
    double f = 0;
    if (live) {
      const int cnt = p.kv_off[s + 1] - p.kv_off[s];
      for (int v = p.kv_off[s]; v < p.kv_off[s + 1]; ++v) {
        const int4 n = p.kv[v];
        f += cos(p.two_pi_over_l * (n.x * dx + n.y * dy + n.z * dz));
      }
      f /= cnt;
    }
    double sf = block_sum(f);
    if (threadIdx.x == 0) atomicAdd(p.fs + (int64_t)g * p.n_shells + s, sf);
  }
}

void ensure_fp64(amdat_ctx* ctx);

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct ShellSet {
  int mode = 0;             // 1 list, 2 octant
  std::vector<int4> kv;     // vectors or octant representatives
  std::vector<int32_t> off; // [n + 1]
  std::vector<float> inv_count;
  int nmax = 0;
};

// Octant reduction of shells that are closed under sign flips of each
// component; returns false when some shell is not (then list mode is used).
static bool octant_shells(const int32_t* off, const int32_t* kvec, int n_shells, ShellSet& out) {
  out.kv.clear();
  out.off.assign(1, 0);
  out.inv_count.clear();
  out.nmax = 0;
  for (int s = 0; s < n_shells; ++s) {
    std::map<std::array<int, 3>, int> seen;
    for (int v = off[s]; v < off[s + 1]; ++v) seen[{kvec[3 * v], kvec[3 * v + 1], kvec[3 * v + 2]}]++;
    for (auto& kvp : seen) {
      if (kvp.second != 1) return false;
      const auto& n = kvp.first;
      for (int m = 1; m < 8; ++m) {
        std::array<int, 3> q = {(m & 1) ? -n[0] : n[0], (m & 2) ? -n[1] : n[1], (m & 4) ? -n[2] : n[2]};
        if (!seen.count(q)) return false;
      }
    }
    for (auto& kvp : seen) {
      const auto& n = kvp.first;
      if (n[0] < 0 || n[1] < 0 || n[2] < 0) continue;
      const int w = (n[0] ? 2 : 1) * (n[1] ? 2 : 1) * (n[2] ? 2 : 1);
      out.kv.push_back(make_int4(n[0], n[1], n[2], w));
      out.nmax = std::max(out.nmax, std::max(n[0], std::max(n[1], n[2])));
    }
    out.off.push_back((int32_t)out.kv.size());
    const int cnt = off[s + 1] - off[s];
    out.inv_count.push_back(cnt ? 1.0f / (float)cnt : 0.0f);
  }
  // each representative as the F_s kernel reads it: its three offsets into the
  // per-thread cosine tables ([axis][n][thread] of FS_THREADS threads) and its
  // multiplicity as FP32 bits
  const int stride = (out.nmax + 1) * FS_THREADS;
  for (auto& r : out.kv) {
    const float w = (float)r.w;
    int32_t wbits;
    std::memcpy(&wbits, &w, 4);
    r = make_int4(r.x * FS_THREADS, stride + r.y * FS_THREADS, 2 * stride + r.z * FS_THREADS, wbits);
  }
  out.mode = 2;
  return true;
}

static void list_shells(const int32_t* off, const int32_t* kvec, int n_shells, ShellSet& out) {
  out.kv.clear();
  out.off.assign(1, 0);
  out.inv_count.clear();
  for (int s = 0; s < n_shells; ++s) {
    for (int v = off[s]; v < off[s + 1]; ++v)
      out.kv.push_back(make_int4(kvec[3 * v], kvec[3 * v + 1], kvec[3 * v + 2], 0));
    out.off.push_back((int32_t)out.kv.size());
    const int cnt = off[s + 1] - off[s];
    out.inv_count.push_back(cnt ? 1.0f / (float)cnt : 0.0f);
  }
  out.mode = 1;
}

static void check_request(amdat_ctx* ctx, const amdat_disp_request* r) {
  AMDAT_REQUIRE(r != nullptr, "null request");
  if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
  AMDAT_REQUIRE(r->precision == AMDAT_MIXED || r->precision == AMDAT_PLAIN_FP64, "bad precision");
  AMDAT_REQUIRE(r->n_shells >= 0 && r->n_bins >= 0, "negative shell or bin count");
  if (r->n_shells > 0) {
    AMDAT_REQUIRE(r->shell_offsets && r->kvec_n, "F_s requested without vectors");
    AMDAT_REQUIRE(r->kvec_period > 0.0f, "kvec_period must be positive");
    AMDAT_REQUIRE(r->shell_offsets[0] == 0, "shell_offsets[0] must be 0");
    for (int s = 0; s < r->n_shells; ++s)
      AMDAT_REQUIRE(r->shell_offsets[s + 1] >= r->shell_offsets[s], "shell_offsets must ascend");
    const int nk = r->shell_offsets[r->n_shells];
    for (int i = 0; i < 3 * nk; ++i)
      AMDAT_REQUIRE(std::abs(r->kvec_n[i]) < (1 << 20), "lattice index too large");
  }
  if (r->n_bins > 0) {
    AMDAT_REQUIRE(r->bin_max > 0.0f, "bin_max must be positive");
    AMDAT_REQUIRE(r->n_bins <= 16384, "at most 16384 G_s bins");
  }
}

template <class T>
static void to_out(amdat_ctx* ctx, T* dst, const T* dev_src, size_t n, int32_t flags) {
  if (!dst || n == 0) return;
  AMDAT_CUDA(cudaMemcpyAsync(dst, dev_src, n * sizeof(T),
                             flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice
                                                       : cudaMemcpyDeviceToHost,
                             ctx->stream));
}

// ---------------------------------------------------------------------------
// plain FP64 path (one list, direct kernels)
// ---------------------------------------------------------------------------
static void disp_plain(amdat_ctx* ctx, const amdat_disp_request* req, int32_t out_flags,
                       double* sum_d2, double* sum_d4, int64_t* atom_pairs, double* fs_sum,
                       int64_t* gs_counts) {
  const PairTable& P = pair_table(ctx, req->fullblock != 0, false);
  const int G = P.n_gaps, S = req->n_shells, NB = req->n_bins;
  const ListEntry& e = list_entry(ctx, req->list);
  ensure_fp64(ctx);
  const size_t n_lg = (size_t)G;
  ShellSet sh;
  if (S) list_shells(req->shell_offsets, req->kvec_n, S, sh);
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t o = 0;
  const size_t o_d2 = o; o = align(o + n_lg * 8);
  const size_t o_d4 = o; o = align(o + n_lg * 8);
  const size_t o_fs = o; o = align(o + n_lg * std::max(S, 1) * 8);
  const size_t o_gs = o; o = align(o + n_lg * std::max(NB, 1) * 8);
  const size_t o_kv = o; o = align(o + std::max<size_t>(sh.kv.size(), 1) * sizeof(int4));
  const size_t o_off = o; o = align(o + std::max<size_t>(sh.off.size(), 1) * 4);
  unsigned char* base = ctx->scratch.reserve(o);
  AMDAT_CUDA(cudaMemsetAsync(base, 0, o_kv, ctx->stream));
  if (S) {
    AMDAT_CUDA(cudaMemcpyAsync(base + o_kv, sh.kv.data(), sh.kv.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
    AMDAT_CUDA(cudaMemcpyAsync(base + o_off, sh.off.data(), sh.off.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  PlainParams pp{};
  pp.u = ctx->u64.ptr;
  pp.n_pad = ctx->n_pad;
  pp.t0 = P.t0.ptr;
  pp.t1 = P.t1.ptr;
  pp.gap = P.gap.ptr;
  pp.n_pairs = P.n_pairs;
  pp.list = ListDev{e.n, e.first, e.contiguous ? nullptr : e.idx.ptr};
  pp.blocks_per_pair = (int32_t)std::max<int64_t>(1, ceil_div(e.n, 256));
  pp.d2 = (double*)(base + o_d2);
  pp.d4 = (double*)(base + o_d4);
  pp.fs = (double*)(base + o_fs);
  pp.n_shells = S;
  pp.kv = (const int4*)(base + o_kv);
  pp.kv_off = (const int32_t*)(base + o_off);
  pp.two_pi_over_l = S ? 6.283185307179586476925286766559 / (double)req->kvec_period : 0.0;
  pp.gs = (unsigned long long*)(base + o_gs);
  pp.n_bins = NB;
  pp.bin_size = NB ? (double)(req->bin_max / (float)NB) : 1.0;
  const int64_t blocks = P.n_pairs * pp.blocks_per_pair;
  if (blocks > 0 && e.n > 0) {
    KernelTimer kt(ctx, "disp_plain_kernel");
    disp_plain_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(pp);
    check_launch("disp_plain_kernel");
    count_launch(ctx);
  }
  to_out(ctx, sum_d2, pp.d2, n_lg, out_flags);
  to_out(ctx, sum_d4, pp.d4, n_lg, out_flags);
  if (S) to_out(ctx, fs_sum, pp.fs, n_lg * S, out_flags);
  if (NB) to_out(ctx, (unsigned long long*)gs_counts, pp.gs, n_lg * NB, out_flags);
  if (atom_pairs) {
    std::vector<int64_t> c(G);
    for (int g = 0; g < G; ++g) c[g] = (int64_t)e.n * (P.gap_first[g + 1] - P.gap_first[g]);
    if (out_flags == AMDAT_OUT_DEVICE)
      AMDAT_CUDA(cudaMemcpyAsync(atom_pairs, c.data(), G * 8, cudaMemcpyHostToDevice, ctx->stream));
    else
      std::memcpy(atom_pairs, c.data(), G * 8);
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace amdat

// ---------------------------------------------------------------------------
// prepared displacement plans (mixed path): device tables built once, a run is
// pure stream work (memsets + persistent kernel + finalize per shell pass),
// optionally captured in a CUDA graph; tile choice optionally autotuned
// ---------------------------------------------------------------------------
struct amdat_disp_plan {
  int n_lists = 0, G = 0, S = 0, NB = 0, n_passes = 1, n_out = 2;
  bool fullblock = false;
  uint64_t scheme_serial = 0;  // time scheme the descriptors were made for
  const float* traj_u = nullptr;  // trajectory storage and shape the plan reads
  int32_t traj_atoms = 0, traj_frames = 0, traj_pad = 0;
  float bin_max = 0.f, period = 1.f;
  amdat::ShellSet sh;
  std::vector<int32_t> lsize;
  std::vector<int64_t> pairs;  // atom_pairs [list][gap]
  // work units: the lists themselves, or membership classes shared by lists
  bool classes = false;
  int n_units = 0;
  std::vector<int32_t> usize;
  std::vector<amdat::ListDev> udev;
  std::vector<int32_t> lu_off, lu_units;  // list -> its units (CSR, ascending)
  amdat::DevBuf<int32_t> class_idx;       // atoms of gathered classes
  int chunk = 0, blocks_per_sm = 0, n_items = 0;
  double tuned_ms = 0.0;
  bool bulk = false;  // MSD + NGP through the bulk-copy-staged kernel
  // device: [descriptors | pair frames | item_first | counters | kv | off | inv | lu_off | lu_units |
  //          part | unit d2 | d4 | fs | gs | list d2 | d4 | fs | gs]
  amdat::DevBuf<unsigned char> dev;
  size_t o_desc = 0, o_frames = 0, o_first = 0, o_counter = 0, o_kv = 0, o_off = 0,
         o_inv = 0, o_luo = 0, o_luu = 0, o_part = 0, o_ud2 = 0, o_ud4 = 0, o_ufs = 0, o_ugs = 0,
         o_d2 = 0, o_d4 = 0, o_fs = 0, o_gs = 0, bytes = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~amdat_disp_plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

namespace amdat {

static void plan_tables(amdat_ctx* ctx, amdat_disp_plan& pl, const PairTable& P, int chunk,
                        int blocks_per_sm) {
  const int G = pl.G;
  const size_t n_ug = (size_t)pl.n_units * G, n_lg = (size_t)pl.n_lists * G;
  std::vector<DispItem> items;
  std::vector<int32_t> item_first(n_ug + 1, 0);
  std::vector<int64_t> key;  // schedule key per item: (unit, chunk, pair)
  // moments-only passes give a unit smaller than half a chunk several pairs
  // of one gap per item (the finalize sums a (unit, gap)'s items anyway), so
  // small lists do not pay one item's fixed cost per pair
  const bool multi_pair = pl.S == 0 && pl.NB == 0;
  for (int u = 0; u < pl.n_units; ++u) {
    const int nch = (int)std::max<int64_t>(1, ceil_div(pl.usize[u], chunk));
    const int ppi = (multi_pair && pl.usize[u] > 0 && 2 * pl.usize[u] <= chunk)
                        ? std::min(MAX_PAIRS_PER_ITEM, chunk / pl.usize[u])
                        : 1;
    for (int g = 0; g < G; ++g) {
      item_first[(size_t)u * G + g] = (int32_t)items.size();
      if (pl.usize[u] == 0) continue;
      for (int pr = P.gap_first[g]; pr < P.gap_first[g + 1]; pr += ppi) {
        const int np = std::min(ppi, P.gap_first[g + 1] - pr);
        for (int c = 0; c < nch; ++c) {
          const int a0 = (int)((int64_t)pl.usize[u] * c / nch);
          const int a1 = (int)((int64_t)pl.usize[u] * (c + 1) / nch);
          items.push_back(DispItem{u, pr, a0, a1, np});
          key.push_back(((int64_t)u << 40) | ((int64_t)c << 20) | (int64_t)pr);
        }
      }
    }
  }
  item_first[n_ug] = (int32_t)items.size();
  // process all pairs of one (unit, atom chunk) together: the chunk's frames
  // are read from HBM once and reused from L2 by the other pairs
  std::vector<int32_t> sched(items.size());
  for (size_t i = 0; i < sched.size(); ++i) sched[i] = (int32_t)i;
  std::stable_sort(sched.begin(), sched.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  // descriptors in processing order (the pair table's frames resolved here)
  const std::vector<int32_t>&ht0 = P.h_t0, &ht1 = P.h_t1, &hgap = P.h_gap;
  std::vector<DispDesc> desc(items.size());
  std::vector<int2> frames;
  for (size_t k = 0; k < sched.size(); ++k) {
    const DispItem& it = items[sched[k]];
    const ListDev& L = pl.udev[it.list];
    desc[k] = DispDesc{sched[k], it.list, it.a0, it.a1, ht0[it.pair], ht1[it.pair],
                       hgap[it.pair], L.first, L.idx, it.n_pairs, (int32_t)frames.size()};
    if (it.n_pairs > 1)
      for (int i = 0; i < it.n_pairs; ++i) frames.push_back(make_int2(ht0[it.pair + i], ht1[it.pair + i]));
  }
  pl.n_items = (int)items.size();
  pl.chunk = chunk;
  pl.blocks_per_sm = blocks_per_sm;
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t S1 = (size_t)std::max(pl.S, 1), NB1 = (size_t)std::max(pl.NB, 1);
  size_t o = 0;
  pl.o_desc = o; o = align(o + std::max<size_t>(desc.size(), 1) * sizeof(DispDesc));
  pl.o_frames = o; o = align(o + std::max<size_t>(frames.size(), 1) * sizeof(int2));
  pl.o_first = o; o = align(o + item_first.size() * 4);
  pl.o_counter = o; o = align(o + 4 * ((size_t)pl.n_passes + 1));  // work counters, then an error word
  pl.o_kv = o; o = align(o + std::max<size_t>(pl.sh.kv.size(), 1) * sizeof(int4));
  pl.o_off = o; o = align(o + std::max<size_t>(pl.sh.off.size(), 1) * 4);
  pl.o_inv = o; o = align(o + std::max<size_t>(pl.sh.inv_count.size(), 1) * 4);
  pl.o_luo = o; o = align(o + std::max<size_t>(pl.lu_off.size(), 1) * 4);
  pl.o_luu = o; o = align(o + std::max<size_t>(pl.lu_units.size(), 1) * 4);
  pl.o_part = o; o = align(o + (size_t)std::max(pl.n_items, 1) * pl.n_out * 8);
  pl.o_ud2 = o; o = align(o + n_ug * 8);
  pl.o_ud4 = o; o = align(o + n_ug * 8);
  pl.o_ufs = o; o = align(o + n_ug * S1 * 8);
  pl.o_ugs = o; o = align(o + n_ug * NB1 * 8);
  if (pl.classes) {
    pl.o_d2 = o; o = align(o + n_lg * 8);
    pl.o_d4 = o; o = align(o + n_lg * 8);
    pl.o_fs = o; o = align(o + n_lg * S1 * 8);
    pl.o_gs = o; o = align(o + n_lg * NB1 * 8);
  } else {
    pl.o_d2 = pl.o_ud2;
    pl.o_d4 = pl.o_ud4;
    pl.o_fs = pl.o_ufs;
    pl.o_gs = pl.o_ugs;
  }
  pl.bytes = o;
  unsigned char* base = pl.dev.reserve(o);
  std::vector<unsigned char> host(pl.o_part, 0);
  std::memcpy(host.data() + pl.o_desc, desc.data(), desc.size() * sizeof(DispDesc));
  std::memcpy(host.data() + pl.o_frames, frames.data(), frames.size() * sizeof(int2));
  std::memcpy(host.data() + pl.o_first, item_first.data(), item_first.size() * 4);
  if (pl.S) {
    std::memcpy(host.data() + pl.o_kv, pl.sh.kv.data(), pl.sh.kv.size() * sizeof(int4));
    std::memcpy(host.data() + pl.o_off, pl.sh.off.data(), pl.sh.off.size() * 4);
    std::memcpy(host.data() + pl.o_inv, pl.sh.inv_count.data(), pl.sh.inv_count.size() * 4);
  }
  if (pl.classes) {
    std::memcpy(host.data() + pl.o_luo, pl.lu_off.data(), pl.lu_off.size() * 4);
    std::memcpy(host.data() + pl.o_luu, pl.lu_units.data(), pl.lu_units.size() * 4);
  }
  AMDAT_CUDA(cudaMemcpyAsync(base, host.data(), pl.o_part, cudaMemcpyHostToDevice, ctx->stream));
  AMDAT_CUDA(cudaMemsetAsync(base + pl.o_ud2, 0, o - pl.o_ud2, ctx->stream));
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
}

// every device operation of one run, in stream order (capturable)
static void plan_launch(amdat_ctx* ctx, amdat_disp_plan& pl, const PairTable& P) {
  unsigned char* base = pl.dev.ptr;
  const size_t n_ug = (size_t)pl.n_units * pl.G, n_lg = (size_t)pl.n_lists * pl.G;
  if (pl.NB) AMDAT_CUDA(cudaMemsetAsync(base + pl.o_ugs, 0, n_ug * pl.NB * 8, ctx->stream));
  if (pl.n_items == 0) {
    AMDAT_CUDA(cudaMemsetAsync(base + pl.o_ud2, 0, pl.bytes - pl.o_ud2, ctx->stream));
    return;
  }
  AMDAT_CUDA(cudaMemsetAsync(base + pl.o_counter, 0, 4 * ((size_t)pl.n_passes + 1), ctx->stream));
  for (int pass = 0; pass < pl.n_passes; ++pass) {
    const int s0 = pass * MAX_FS;
    const int nfs = pl.S ? std::min(MAX_FS, pl.S - s0) : 0;
    DispParams p{};
    p.u = ctx->u.ptr;
    p.n_pad = ctx->n_pad;
    p.desc = (const DispDesc*)(base + pl.o_desc);
    p.frames = (const int2*)(base + pl.o_frames);
    p.n_items = pl.n_items;
    p.counter = (int32_t*)(base + pl.o_counter) + pass;
    p.part = (double*)(base + pl.o_part);
    p.n_out = pl.n_out;
    p.want_moments = pass == 0;
    p.gs = (unsigned long long*)(base + pl.o_ugs);
    p.n_gaps = pl.G;
    p.n_bins = pass == 0 ? pl.NB : 0;
    p.bin_size = pl.NB ? pl.bin_max / (float)pl.NB : 1.0f;
    p.n_fs = nfs;
    p.fs_mode = pl.S ? pl.sh.mode : 0;
    p.kv = (const int4*)(base + pl.o_kv);
    p.kv_off = (const int32_t*)(base + pl.o_off) + s0;
    p.inv_count = (const float*)(base + pl.o_inv) + s0;
    p.nmax = pl.sh.nmax;
    p.period = pl.S ? pl.period : 1.0f;
    const bool gs = p.n_bins > 0;
    const int mode = nfs ? pl.sh.mode : 0;
    const int threads = mode ? FS_THREADS : DISP_THREADS;
    size_t shm = gs ? (size_t)((pl.NB + 3) & ~3) * 4 : 0;
    if (mode == 2) shm += (size_t)3 * (pl.sh.nmax + 1) * threads * 4;
    if (mode != 0) {
      // the pass's vectors / representatives in shared memory when they take at most 32 KB
      const int n_rep = pl.sh.off[s0 + nfs] - pl.sh.off[s0];
      if (n_rep <= 2048) {
        p.n_rep_smem = n_rep;
        shm += (size_t)n_rep * sizeof(int4);
      }
    }
    auto launch = [&](auto kernel) {
      if (shm > 48 * 1024)
        AMDAT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
      static thread_local std::map<std::pair<const void*, size_t>, int> occ_cache;
      const auto okey = std::make_pair((const void*)kernel, shm);
      int occ = 0;
      auto oit = occ_cache.find(okey);
      if (oit != occ_cache.end()) {
        occ = oit->second;
      } else {
        AMDAT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, shm));
        occ_cache[okey] = occ;
      }
      const int bps = std::max(1, std::min(occ, pl.blocks_per_sm));
      const int grid = (int)std::min<int64_t>((int64_t)bps * ctx->n_sm, pl.n_items);
      KernelTimer kt(ctx, "disp_mixed_kernel");
      kernel<<<grid, threads, shm, ctx->stream>>>(p);
      check_launch("disp_mixed_kernel");
      count_launch(ctx);
    };
    if (mode == 0 && !gs && pl.bulk) {
      auto bulk = [&](auto kernel, size_t smem_bytes, int per_sm) {
        const size_t bshm = smem_bytes + 128;
        AMDAT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bshm));
        const int grid = (int)std::min<int64_t>((int64_t)per_sm * ctx->n_sm, pl.n_items);
        KernelTimer kt(ctx, "disp_bulk_kernel");
        kernel<<<grid, BK_THREADS, bshm, ctx->stream>>>(p, (int*)(base + pl.o_counter) + pl.n_passes);
        check_launch("disp_bulk_kernel");
        count_launch(ctx);
      };
      // 512-atom segments, 4 stages, 4 blocks per SM: the fastest of the ring
      // shapes measured (2048 x 4 x 1, 1024 x 8 x 1, 1024 x 4 x 2, 512 x 8 x 2
      // were slower; each block's single producer thread paces its ring)
      bulk(disp_bulk_kernel<512, 4>, sizeof(BkSmem<512, 4>), 4);
    } else if (mode == 0) {
      if (gs) launch(disp_mixed_kernel<0, true>); else launch(disp_mixed_kernel<0, false>);
    }
    else if (mode == 1) { if (gs) launch(disp_mixed_kernel<1, true>); else launch(disp_mixed_kernel<1, false>); }
    else { if (gs) launch(disp_mixed_kernel<2, true>); else launch(disp_mixed_kernel<2, false>); }
    disp_finalize_kernel<<<(unsigned)ceil_div((int64_t)n_ug * (2 + nfs), 8), 256, 0, ctx->stream>>>(
        p.part, pl.n_out, (const int32_t*)(base + pl.o_first), (int32_t)n_ug,
        pass == 0 ? (double*)(base + pl.o_ud2) : nullptr, pass == 0 ? (double*)(base + pl.o_ud4) : nullptr,
        pl.S ? (double*)(base + pl.o_ufs) : nullptr, std::max(pl.S, 1), s0, nfs, pass == 0 ? 1 : 0);
    check_launch("disp_finalize_kernel");
    count_launch(ctx);
  }
  if (pl.classes) {
    disp_combine_kernel<<<(unsigned)ceil_div((int64_t)n_lg * (2 + pl.S), 8), 256, 0, ctx->stream>>>(
        pl.G, pl.S, (int32_t)n_lg, (const int32_t*)(base + pl.o_luo), (const int32_t*)(base + pl.o_luu),
        (const double*)(base + pl.o_ud2), (const double*)(base + pl.o_ud4), (const double*)(base + pl.o_ufs),
        (double*)(base + pl.o_d2), (double*)(base + pl.o_d4), (double*)(base + pl.o_fs));
    check_launch("disp_combine_kernel");
    count_launch(ctx);
    if (pl.NB) {
      disp_combine_gs_kernel<<<(unsigned)n_lg, 128, 0, ctx->stream>>>(
          pl.G, pl.NB, (const int32_t*)(base + pl.o_luo), (const int32_t*)(base + pl.o_luu),
          (const unsigned long long*)(base + pl.o_ugs), (unsigned long long*)(base + pl.o_gs));
      check_launch("disp_combine_gs_kernel");
      count_launch(ctx);
    }
  }
}

// ---- autotuner cache: JSON lines {"key": ..., "chunk": c, "blocks_per_sm": b, "ms": t}
static std::map<std::string, std::pair<int, int>>& tune_cache() {
  static std::map<std::string, std::pair<int, int>> c;
  static bool loaded = false;
  if (!loaded) {
    loaded = true;
    if (const char* f = std::getenv("AMDAT_TUNE_CACHE")) {
      FILE* fp = std::fopen(f, "r");
      if (fp) {
        char line[512], key[256];
        int ch = 0, bps = 0;
        while (std::fgets(line, sizeof(line), fp))
          if (std::sscanf(line, "{\"key\": \"%255[^\"]\", \"chunk\": %d, \"blocks_per_sm\": %d", key, &ch, &bps) == 3)
            c[key] = {ch, bps};
        std::fclose(fp);
      }
    }
  }
  return c;
}

static void tune_store(const std::string& key, int ch, int bps, double ms) {
  tune_cache()[key] = {ch, bps};
  if (const char* f = std::getenv("AMDAT_TUNE_CACHE")) {
    FILE* fp = std::fopen(f, "a");
    if (fp) {
      std::fprintf(fp, "{\"key\": \"%s\", \"chunk\": %d, \"blocks_per_sm\": %d, \"ms\": %.6f}\n",
                   key.c_str(), ch, bps, ms);
      std::fclose(fp);
    }
  }
}

// Membership classes of a plan's lists: atoms that belong to exactly the same
// lists form one class.  Adopted when the classes stream at most 4/5 of the
// lists' atoms and there are at most four classes per list; otherwise the
// lists stay the work units.
static void plan_classes(amdat_ctx* ctx, amdat_disp_plan& pl, const int32_t* lists) {
  const int L = pl.n_lists;
  const int words = (L + 63) / 64;
  const int64_t N = ctx->n_atoms;
  int64_t list_atoms = 0;
  for (int l = 0; l < L; ++l) list_atoms += pl.lsize[l];
  if (list_atoms == 0) return;
  std::vector<uint64_t> mask((size_t)N * words, 0ull);
  std::vector<int32_t> buf;
  for (int l = 0; l < L; ++l) {
    const ListEntry& e = list_entry(ctx, lists[l]);
    if (e.n == 0) continue;
    const int32_t* a = nullptr;
    if (!e.contiguous) {
      buf.resize(e.n);
      AMDAT_CUDA(cudaMemcpy(buf.data(), e.idx.ptr, (size_t)e.n * 4, cudaMemcpyDeviceToHost));
      a = buf.data();
    }
    for (int i = 0; i < e.n; ++i) {
      const int64_t atom = a ? a[i] : (int64_t)e.first + i;
      mask[(size_t)atom * words + l / 64] |= 1ull << (l % 64);
    }
  }
  std::vector<int32_t> members;
  for (int64_t a = 0; a < N; ++a)
    for (int w = 0; w < words; ++w)
      if (mask[(size_t)a * words + w]) {
        members.push_back((int32_t)a);
        break;
      }
  auto less = [&](int32_t x, int32_t y) {
    for (int w = words - 1; w >= 0; --w) {
      const uint64_t mx = mask[(size_t)x * words + w], my = mask[(size_t)y * words + w];
      if (mx != my) return mx < my;
    }
    return x < y;
  };
  std::sort(members.begin(), members.end(), less);
  auto same = [&](int32_t x, int32_t y) {
    for (int w = 0; w < words; ++w)
      if (mask[(size_t)x * words + w] != mask[(size_t)y * words + w]) return false;
    return true;
  };
  std::vector<int32_t> start;
  for (size_t i = 0; i < members.size(); ++i)
    if (i == 0 || !same(members[i - 1], members[i])) start.push_back((int32_t)i);
  const int n_cls = (int)start.size();
  start.push_back((int32_t)members.size());
  if ((int64_t)members.size() * 5 > list_atoms * 4 || n_cls > 4 * L) return;
  // adopt: class atoms ascending (members are sorted by mask, then atom)
  pl.classes = true;
  pl.n_units = n_cls;
  pl.usize.assign(n_cls, 0);
  pl.udev.assign(n_cls, ListDev{0, 0, nullptr});
  pl.class_idx.reserve(std::max<size_t>(members.size(), 1));
  AMDAT_CUDA(cudaMemcpy(pl.class_idx.ptr, members.data(), members.size() * 4, cudaMemcpyHostToDevice));
  std::vector<std::vector<int32_t>> per_list(L);
  for (int c = 0; c < n_cls; ++c) {
    const int32_t b = start[c], e = start[c + 1];
    pl.usize[c] = e - b;
    const bool contiguous = members[e - 1] - members[b] == e - 1 - b;
    pl.udev[c] = contiguous ? ListDev{e - b, members[b], nullptr} : ListDev{e - b, 0, pl.class_idx.ptr + b};
    const int32_t rep = members[b];
    for (int l = 0; l < L; ++l)
      if (mask[(size_t)rep * words + l / 64] >> (l % 64) & 1ull) per_list[l].push_back(c);
  }
  pl.lu_off.assign(L + 1, 0);
  pl.lu_units.clear();
  for (int l = 0; l < L; ++l) {
    pl.lu_off[l] = (int32_t)pl.lu_units.size();
    pl.lu_units.insert(pl.lu_units.end(), per_list[l].begin(), per_list[l].end());
  }
  pl.lu_off[L] = (int32_t)pl.lu_units.size();
}

static amdat_disp_plan* plan_create(amdat_ctx* ctx, const amdat_disp_request* req,
                                    const int32_t* lists, int32_t n_lists, int32_t flags) {
  check_request(ctx, req);
  AMDAT_REQUIRE(req->precision == AMDAT_MIXED, "plans run the mixed-precision path");
  AMDAT_REQUIRE(lists != nullptr && n_lists >= 1, "need >= 1 list");
  const PairTable& P = pair_table(ctx, req->fullblock != 0, false);
  auto* pl = new amdat_disp_plan();
  try {
    pl->n_lists = n_lists;
    pl->G = P.n_gaps;
    pl->S = req->n_shells;
    pl->NB = req->n_bins;
    pl->fullblock = req->fullblock != 0;
    pl->scheme_serial = ctx->scheme_serial;
    pl->traj_u = ctx->u.ptr;
    pl->traj_atoms = ctx->n_atoms;
    pl->traj_frames = ctx->n_frames;
    pl->traj_pad = ctx->n_pad;
    pl->bin_max = req->bin_max;
    pl->period = req->kvec_period;
    if (pl->S) {
      if (!octant_shells(req->shell_offsets, req->kvec_n, pl->S, pl->sh) || pl->sh.nmax > 48)
        list_shells(req->shell_offsets, req->kvec_n, pl->S, pl->sh);
    }
    pl->n_passes = pl->S ? (int)ceil_div(pl->S, MAX_FS) : 1;
    pl->n_out = 2 + (pl->S ? std::min(pl->S, MAX_FS) : 0);
    int64_t total_atoms = 0;
    for (int l = 0; l < n_lists; ++l) {
      const ListEntry& e = list_entry(ctx, lists[l]);
      pl->udev.push_back(ListDev{e.n, e.first, e.contiguous ? nullptr : e.idx.ptr});
      pl->lsize.push_back(e.n);
      pl->usize.push_back(e.n);
      total_atoms += e.n;
    }
    pl->n_units = n_lists;
    if (n_lists > 1 && !(flags & AMDAT_PLAN_NO_SHARING)) plan_classes(ctx, *pl, lists);
    int64_t unit_atoms = 0;
    for (int u = 0; u < pl->n_units; ++u) unit_atoms += pl->usize[u];
    pl->pairs.assign((size_t)n_lists * pl->G, 0);
    for (int l = 0; l < n_lists; ++l)
      for (int g = 0; g < pl->G; ++g)
        pl->pairs[(size_t)l * pl->G + g] = (int64_t)pl->lsize[l] * (P.gap_first[g + 1] - P.gap_first[g]);
    // MSD + NGP with contiguous members may run the bulk-copy-staged kernel
    // (AMDAT_DISP_KERNEL=bulk at plan creation)
    {
      const char* kern = std::getenv("AMDAT_DISP_KERNEL");
      bool contiguous = true;
      for (const ListDev& u : pl->udev) contiguous = contiguous && u.idx == nullptr;
      pl->bulk = kern && std::strcmp(kern, "bulk") == 0 && pl->S == 0 && pl->NB == 0 && contiguous;
    }
    // default tile: full chunks stream memory; F_s or few pairs want smaller
    // chunks to keep every SM busy
    const int64_t want_items = (int64_t)ctx->n_sm * 16;
    int64_t chunk = DISP_CHUNK;
    if (P.n_pairs > 0 && unit_atoms > 0)
      chunk = std::max<int64_t>(pl->S ? 128 : 1024,
                                std::min<int64_t>(DISP_CHUNK, ceil_div(unit_atoms * P.n_pairs, want_items)));
    // list-mode F_s holds few registers and only its vectors in shared memory:
    // more resident blocks hide the latency of its cosine chain
    int bps = pl->S ? (pl->sh.mode == 1 ? 8 : 4) : 8;
    char keybuf[256];
    std::snprintf(keybuf, sizeof(keybuf), "sm%d_mode%d%s_S%d_NB%d_L%d_U%d_atoms%lld_unit%lld_pairs%lld",
                  ctx->n_sm, pl->S ? pl->sh.mode : 0, pl->bulk ? "b" : "", pl->S, pl->NB, n_lists, pl->n_units,
                  (long long)total_atoms, (long long)unit_atoms, (long long)P.n_pairs);
    const std::string key(keybuf);
    auto hit = tune_cache().find(key);
    if (hit != tune_cache().end()) {
      chunk = hit->second.first;
      bps = hit->second.second;
    } else if (flags & AMDAT_PLAN_AUTOTUNE) {
      // time each candidate (warm-up + 3 runs, CUDA events) and keep the fastest
      // candidates: F_s is compute bound (small chunks, fewer heavier blocks);
      // MSD-only streams memory (large chunks, more resident blocks)
      const std::vector<int> chunks = pl->S ? std::vector<int>{256, 512, 1024, 2048}
                                            : std::vector<int>{1024, 2048, 4096, 8192};
      const std::vector<int> bpss = pl->S ? (pl->sh.mode == 1 ? std::vector<int>{4, 8, 16} : std::vector<int>{2, 4, 8})
                                          : std::vector<int>{4, 8};
      cudaEvent_t a, b;
      AMDAT_CUDA(cudaEventCreate(&a));
      AMDAT_CUDA(cudaEventCreate(&b));
      double best = 1e30;
      int bc = (int)chunk, bb = bps;
      for (int c : chunks) {
        for (int bp : bpss) {
          plan_tables(ctx, *pl, P, c, bp);
          plan_launch(ctx, *pl, P);
          AMDAT_CUDA(cudaEventRecord(a, ctx->stream));
          for (int r = 0; r < 2; ++r) plan_launch(ctx, *pl, P);
          AMDAT_CUDA(cudaEventRecord(b, ctx->stream));
          AMDAT_CUDA(cudaEventSynchronize(b));
          float ms = 0.f;
          AMDAT_CUDA(cudaEventElapsedTime(&ms, a, b));
          if (ms / 2 < best) {
            best = ms / 2;
            bc = c;
            bb = bp;
          }
        }
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      chunk = bc;
      bps = bb;
      pl->tuned_ms = best;
      tune_store(key, bc, bb, best);
    }
    plan_tables(ctx, *pl, P, (int)chunk, bps);
    if (flags & AMDAT_PLAN_GRAPH) {
      AMDAT_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      const bool prof = ctx->profiling;
      ctx->profiling = false;  // events are not recorded inside a graph
      try {
        plan_launch(ctx, *pl, P);
      } catch (...) {
        ctx->profiling = prof;
        cudaGraph_t g;
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      ctx->profiling = prof;
      AMDAT_CUDA(cudaStreamEndCapture(ctx->stream, &pl->graph));
      AMDAT_CUDA(cudaGraphInstantiate(&pl->exec, pl->graph, 0));
    }
  } catch (...) {
    delete pl;
    throw;
  }
  return pl;
}

static void plan_run(amdat_ctx* ctx, amdat_disp_plan* pl) {
  AMDAT_REQUIRE(pl != nullptr, "null plan");
  if (pl->scheme_serial != ctx->scheme_serial)
    throw Error(AMDAT_ERR_STATE, "the time scheme changed after the plan was made; make a new plan");
  // a re-upload of the same shape keeps the storage and the lists; another
  // shape may move the storage and drops the lists the descriptors point into
  if (pl->traj_u != ctx->u.ptr || pl->traj_atoms != ctx->n_atoms || pl->traj_frames != ctx->n_frames ||
      pl->traj_pad != ctx->n_pad)
    throw Error(AMDAT_ERR_STATE, "a trajectory of another shape was uploaded after the plan was made; make a new plan");
  const PairTable& P = pair_table(ctx, pl->fullblock, false);
  if (pl->exec) {
    KernelTimer kt(ctx, "disp_plan_graph");
    AMDAT_CUDA(cudaGraphLaunch(pl->exec, ctx->stream));
    count_launch(ctx, 2 * pl->n_passes);
  } else {
    plan_launch(ctx, *pl, P);
  }
}

static void plan_read(amdat_ctx* ctx, amdat_disp_plan* pl, int32_t out_flags, double* sum_d2,
                      double* sum_d4, int64_t* atom_pairs, double* fs_sum, int64_t* gs_counts) {
  AMDAT_REQUIRE(out_flags == AMDAT_OUT_HOST || out_flags == AMDAT_OUT_DEVICE, "bad out_flags");
  const size_t n_lg = (size_t)pl->n_lists * pl->G;
  unsigned char* base = pl->dev.ptr;
  to_out(ctx, sum_d2, (const double*)(base + pl->o_d2), n_lg, out_flags);
  to_out(ctx, sum_d4, (const double*)(base + pl->o_d4), n_lg, out_flags);
  if (pl->S) to_out(ctx, fs_sum, (const double*)(base + pl->o_fs), n_lg * pl->S, out_flags);
  if (pl->NB) to_out(ctx, (unsigned long long*)gs_counts, (const unsigned long long*)(base + pl->o_gs), n_lg * pl->NB, out_flags);
  if (atom_pairs) {
    if (out_flags == AMDAT_OUT_DEVICE)
      AMDAT_CUDA(cudaMemcpyAsync(atom_pairs, pl->pairs.data(), n_lg * 8, cudaMemcpyHostToDevice, ctx->stream));
    else
      std::memcpy(atom_pairs, pl->pairs.data(), n_lg * 8);
  }
  if (out_flags == AMDAT_OUT_HOST || atom_pairs || pl->bulk) AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  if (pl->bulk) {
    int err = 0;
    AMDAT_CUDA(cudaMemcpy(&err, base + pl->o_counter + 4 * (size_t)pl->n_passes, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) throw Error(AMDAT_ERR_TIMEOUT, "bulk-staged displacement kernel: a bounded wait timed out");
  }
}

static void disp_run_impl(amdat_ctx* ctx, const amdat_disp_request* req, const int32_t* lists,
                          int32_t n_lists, int32_t out_flags, double* sum_d2, double* sum_d4,
                          int64_t* atom_pairs, double* fs_sum, int64_t* gs_counts) {
  check_request(ctx, req);
  AMDAT_REQUIRE(out_flags == AMDAT_OUT_HOST || out_flags == AMDAT_OUT_DEVICE, "bad out_flags");
  if (req->precision == AMDAT_PLAIN_FP64) {
    AMDAT_REQUIRE(n_lists == 1, "the plain FP64 path runs one list per call");
    amdat_disp_request r = *req;
    r.list = lists[0];
    disp_plain(ctx, &r, out_flags, sum_d2, sum_d4, atom_pairs, fs_sum, gs_counts);
    return;
  }
  // repeated one-shot runs of one request reuse its prepared plan (tables,
  // descriptors and buffers); a new scheme or trajectory clears the cache
  std::string key;
  auto put = [&key](const void* v, size_t n) { key.append(static_cast<const char*>(v), n); };
  put(&ctx->scheme_serial, 8);
  put(&ctx->traj_serial, 8);
  put(&req->fullblock, 4);
  put(&req->n_shells, 4);
  put(&req->kvec_period, 4);
  put(&req->n_bins, 4);
  put(&req->bin_max, 4);
  put(&n_lists, 4);
  put(lists, 4 * (size_t)n_lists);
  if (req->n_shells > 0) {
    put(req->shell_offsets, 4 * (size_t)(req->n_shells + 1));
    put(req->kvec_n, 12 * (size_t)std::max(req->shell_offsets[req->n_shells], 0));
  }
  std::shared_ptr<amdat_disp_plan> pl;
  auto& cache = ctx->disp_cache;
  for (size_t i = 0; i < cache.size(); ++i)
    if (cache[i].first == key) {
      pl = cache[i].second;
      cache.erase(cache.begin() + (std::ptrdiff_t)i);
      break;
    }
  if (!pl) pl.reset(plan_create(ctx, req, lists, n_lists, 0), [](amdat_disp_plan* p) { delete p; });
  cache.emplace_back(std::move(key), pl);
  if (cache.size() > DISP_CACHE_PLANS) cache.erase(cache.begin());
  plan_run(ctx, pl.get());
  plan_read(ctx, pl.get(), out_flags, sum_d2, sum_d4, atom_pairs, fs_sum, gs_counts);
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_disp_run(amdat_ctx* ctx, const amdat_disp_request* req, int32_t out_flags,
                            double* sum_d2, double* sum_d4, int64_t* atom_pairs, double* fs_sum,
                            int64_t* gs_counts) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(req != nullptr, "null request");
    const int32_t l = req->list;
    disp_run_impl(ctx, req, &l, 1, out_flags, sum_d2, sum_d4, atom_pairs, fs_sum, gs_counts);
  });
}

amdat_status amdat_disp_run_lists(amdat_ctx* ctx, const amdat_disp_request* req,
                                  const int32_t* lists, int32_t n_lists, int32_t out_flags,
                                  double* sum_d2, double* sum_d4, int64_t* atom_pairs,
                                  double* fs_sum, int64_t* gs_counts) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(lists != nullptr && n_lists >= 1, "need >= 1 list");
    disp_run_impl(ctx, req, lists, n_lists, out_flags, sum_d2, sum_d4, atom_pairs, fs_sum, gs_counts);
  });
}

amdat_status amdat_disp_plan_create(amdat_ctx* ctx, const amdat_disp_request* req,
                                    const int32_t* lists, int32_t n_lists, int32_t flags,
                                    amdat_disp_plan** plan) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(plan != nullptr, "null plan pointer");
    *plan = plan_create(ctx, req, lists, n_lists, flags);
  });
}

amdat_status amdat_disp_plan_run(amdat_ctx* ctx, amdat_disp_plan* plan) {
  return guarded([&] {
    check_ctx(ctx);
    plan_run(ctx, plan);
  });
}

amdat_status amdat_disp_plan_read(amdat_ctx* ctx, amdat_disp_plan* plan, int32_t out_flags,
                                  double* sum_d2, double* sum_d4, int64_t* atom_pairs,
                                  double* fs_sum, int64_t* gs_counts) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(plan != nullptr, "null plan");
    plan_read(ctx, plan, out_flags, sum_d2, sum_d4, atom_pairs, fs_sum, gs_counts);
  });
}

amdat_status amdat_disp_plan_info(amdat_disp_plan* plan, int32_t* chunk, int32_t* blocks_per_sm,
                                  int64_t* n_items, double* tuned_ms) {
  return guarded([&] {
    AMDAT_REQUIRE(plan != nullptr, "null plan");
    if (chunk) *chunk = plan->chunk;
    if (blocks_per_sm) *blocks_per_sm = plan->blocks_per_sm;
    if (n_items) *n_items = plan->n_items;
    if (tuned_ms) *tuned_ms = plan->tuned_ms;
  });
}

amdat_status amdat_disp_plan_sharing(amdat_disp_plan* plan, int32_t* n_units, int64_t* unit_atoms,
                                     int64_t* list_atoms) {
  return guarded([&] {
    AMDAT_REQUIRE(plan != nullptr, "null plan");
    int64_t ua = 0, la = 0;
    for (int32_t v : plan->usize) ua += v;
    for (int32_t v : plan->lsize) la += v;
    if (n_units) *n_units = plan->n_units;
    if (unit_atoms) *unit_atoms = ua;
    if (list_atoms) *list_atoms = la;
  });
}

amdat_status amdat_disp_plan_destroy(amdat_ctx* ctx, amdat_disp_plan* plan) {
  return guarded([&] {
    if (ctx) {
      check_ctx(ctx);
      AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    delete plan;
  });
}

}  // extern "C"
