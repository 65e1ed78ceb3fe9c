// Pair histograms: the radial distribution function's per-frame pair loop
// (Radial_Distribution_Function::listkernel2 + bin,
// src/radial_distribution_function.cpp:233-253) and the distinct van Hove
// pair loop over time pairs (Van_Hove_Distinct::listkernel2,
// src/van_hove_distinct.cpp:200-213, with the distance the reference meant to
// bin: the minimum-image |r_j(t1) - r_i(t0)|).
//
// Every distance follows the reference's FP32 chain exactly -
// Coordinate::length_unwrapped (src/coordinate.cpp:126-137): per axis
// d = r_j - r_i, m = min(|d|, L - |d|); length = sqrtf((mx*mx + my*my) + mz*mz);
// bin = int(length / bin_size) - with correctly rounded, uncontracted
// operations, so the integer counts equal the reference's bit for bit.
// Pairs whose squared length is safely beyond the last bin skip the square
// root and the division; the others estimate the bin from rsqrtf and take
// the correctly rounded chain only when the estimate lies within its error
// bound of a bin edge.
//
// A block owns 512 members i of list 1 (two per thread, positions in
// registers) and streams list 2 through shared memory in tiles of 1024.  Counts go to per-warp
// shared-memory histograms, then once per block to the global int64
// histogram with integer atomics (exact, order-independent).  For the RDF
// with list1 == list2 the unordered pairs j > i are visited once and counted
// twice (|d| is symmetric to the bit under exchange of i and j).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"

namespace amdat {

constexpr int PH_THREADS = 256;
constexpr int PH_I_PER_BLOCK = 2 * PH_THREADS;  // two list-1 members per thread
constexpr int PH_JT = 1024;

struct PHList {
  int32_t n;
  int32_t first;
  const int32_t* idx;
};

static PHList phview(const ListEntry& e) {
  return PHList{e.n, e.first, e.contiguous ? nullptr : e.idx.ptr};
}

__device__ __forceinline__ int member(const PHList& l, int a) {
  return l.idx ? l.idx[a] : l.first + a;
}

__device__ __forceinline__ float min_image(float d, float L) {
  const float a = fabsf(d);
  const float b = __fsub_rn(L, a);
  return a < b ? a : b;
}

struct PHParams {
  const float* w;
  int64_t n_pad;
  PHList l1, l2;
  const int32_t* frame_a;  // [n_rows] frame of list-1 positions
  const int32_t* frame_b;  // [n_rows] frame of list-2 positions
  const int32_t* row_of;   // [n_rows] output row (frame index or gap)
  int32_t symmetric;       // l1 == l2 and frame_a == frame_b: visit j > i, count 2
  float3 box;
  float bin_size;
  float inv_bin;  // 1 / bin_size (the fast bin estimate)
  float s2_cut;
  int32_t n_bins;
  unsigned long long* counts;  // [rows][n_bins]
};

// one pair: the reference's FP32 minimum-image length and its bin, counted into
// the warp's shared histogram
template <bool SYM>
__device__ __forceinline__ void pair_term(const PHParams& p, float4 c, float xi, float yi, float zi,
                                          unsigned int* hist, unsigned int inc) {
  const float mx = min_image(__fsub_rn(c.x, xi), p.box.x);
  const float my = min_image(__fsub_rn(c.y, yi), p.box.y);
  const float mz = min_image(__fsub_rn(c.z, zi), p.box.z);
  const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my)), __fmul_rn(mz, mz));
  if (s2 < p.s2_cut) {
    // bin = int(sqrt_rn(s2) / bin_size), the reference's chain.  First from
    // rsqrtf (<= 2 ulp) and the reciprocal bin size: within 1e-6 relative of
    // the exact quotient, so its integer part is the exact one unless the
    // quotient lies within that margin of an integer; those pairs (and s2 = 0)
    // take the correctly rounded chain.  (The symmetric RDF pass, where most
    // pairs are in range; the sparse distinct van Hove pass keeps the short
    // exact branch.)
    int b;
    if (SYM) {
      const float x = __fmul_rn(__fmul_rn(s2, rsqrtf(s2)), p.inv_bin);
      b = (int)x;
      const float frac = __fsub_rn(x, (float)b);
      const float margin = fmaf(x, 1e-6f, 1e-6f);
      if (!(s2 > 0.f) || frac <= margin || frac >= 1.f - margin)
        b = (int)__fdiv_rn(__fsqrt_rn(s2), p.bin_size);
    } else {
      b = (int)__fdiv_rn(__fsqrt_rn(s2), p.bin_size);
    }
    if (b >= 0 && b < p.n_bins) atomicAdd(hist + b, inc);
  }
}

// SYM: the symmetric pass (list1 == list2, one frame): j > i, each pair counted
// twice.  A thread holds two members of list 1 (i and i + PH_THREADS) in
// registers, so each staged list-2 position (one 16-byte shared load: x, y, z
// and the atom index) serves two pairs.
template <bool SYM>
__global__ void __launch_bounds__(PH_THREADS)
    pair_hist_kernel(PHParams p) {
  extern __shared__ unsigned int sh_hist[];  // [8 warps][n_bins]
  __shared__ float4 sj[PH_JT];               // x, y, z, atom index bits
  const int q = blockIdx.y;
  const float* A = p.w + (int64_t)p.frame_a[q] * 3 * p.n_pad;
  const float* B = p.w + (int64_t)p.frame_b[q] * 3 * p.n_pad;
  const int warp = threadIdx.x >> 5;
  unsigned int* hist = sh_hist + warp * p.n_bins;
  for (int b = threadIdx.x; b < 8 * p.n_bins; b += blockDim.x) sh_hist[b] = 0u;
  const int i0 = blockIdx.x * PH_I_PER_BLOCK;
  const int ia = i0 + threadIdx.x, ib = ia + PH_THREADS;
  const bool la = ia < p.l1.n, lb = ib < p.l1.n;
  int aa = -1, ab = -1;
  float xa = 0.f, ya = 0.f, za = 0.f, xb = 0.f, yb = 0.f, zb = 0.f;
  if (la) {
    aa = member(p.l1, ia);
    xa = A[aa];
    ya = A[p.n_pad + aa];
    za = A[2 * p.n_pad + aa];
  }
  if (lb) {
    ab = member(p.l1, ib);
    xb = A[ab];
    yb = A[p.n_pad + ab];
    zb = A[2 * p.n_pad + ab];
  }
  const unsigned int inc = SYM ? 2u : 1u;
  const int j_begin = SYM ? i0 : 0;
  __syncthreads();
  for (int j0 = j_begin; j0 < p.l2.n; j0 += PH_JT) {
    const int nj = min(PH_JT, p.l2.n - j0);
    __syncthreads();
    for (int t = threadIdx.x; t < nj; t += blockDim.x) {
      const int aj = member(p.l2, j0 + t);
      sj[t] = make_float4(B[aj], B[p.n_pad + aj], B[2 * p.n_pad + aj], __int_as_float(aj));
    }
    __syncthreads();
    if (!la) continue;  // lb implies la
    // j > i for the symmetric pass (i != j is implied), i != j checked otherwise
    const int t_begin = SYM ? max(0, ia + 1 - j0) : 0;
    const int t_b = SYM ? ib + 1 - j0 : 0;  // the second member's first t
    for (int t = t_begin; t < nj; ++t) {
      const float4 c = sj[t];
      if (SYM || __float_as_int(c.w) != aa) pair_term<SYM>(p, c, xa, ya, za, hist, inc);
      if (lb && (SYM ? t >= t_b : __float_as_int(c.w) != ab)) pair_term<SYM>(p, c, xb, yb, zb, hist, inc);
    }
  }
  __syncthreads();
  unsigned long long* dst = p.counts + (int64_t)p.row_of[q] * p.n_bins;
  for (int b = threadIdx.x; b < p.n_bins; b += blockDim.x) {
    unsigned long long s = 0;
    for (int w = 0; w < 8; ++w) s += sh_hist[w * p.n_bins + b];
    if (s) atomicAdd(dst + b, s);
  }
}

static void run_pair_hist(amdat_ctx* ctx, const ListEntry& l1, const ListEntry& l2, bool symmetric,
                          const std::vector<int32_t>& fa, const std::vector<int32_t>& fb,
                          const std::vector<int32_t>& row, int32_t n_rows_out, float max_distance,
                          int32_t n_bins, int32_t out_flags, int64_t* counts) {
  AMDAT_REQUIRE(n_bins >= 1 && n_bins <= 4096, "n_bins must be in [1, 4096]");
  AMDAT_REQUIRE(max_distance > 0.0f, "max_distance must be positive");
  AMDAT_REQUIRE(counts != nullptr, "null output");
  const size_t n_q = fa.size();
  const size_t n_out = (size_t)n_rows_out * n_bins;
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t o = 0;
  const size_t o_fa = o; o = align(o + std::max<size_t>(n_q, 1) * 4);
  const size_t o_fb = o; o = align(o + std::max<size_t>(n_q, 1) * 4);
  const size_t o_row = o; o = align(o + std::max<size_t>(n_q, 1) * 4);
  const size_t o_cnt = o; o = align(o + n_out * 8);
  unsigned char* base = ctx->scratch.reserve(o);
  std::vector<unsigned char> host(o_cnt, 0);
  if (n_q) {
    std::memcpy(host.data() + o_fa, fa.data(), n_q * 4);
    std::memcpy(host.data() + o_fb, fb.data(), n_q * 4);
    std::memcpy(host.data() + o_row, row.data(), n_q * 4);
  }
  AMDAT_CUDA(cudaMemcpyAsync(base, host.data(), o_cnt, cudaMemcpyHostToDevice, ctx->stream));
  AMDAT_CUDA(cudaMemsetAsync(base + o_cnt, 0, n_out * 8, ctx->stream));
  PHParams p{};
  p.w = ctx->w.ptr;
  p.n_pad = ctx->n_pad;
  p.l1 = phview(l1);
  p.l2 = phview(l2);
  p.frame_a = (const int32_t*)(base + o_fa);
  p.frame_b = (const int32_t*)(base + o_fb);
  p.row_of = (const int32_t*)(base + o_row);
  p.symmetric = symmetric ? 1 : 0;
  p.box = make_float3(ctx->box[0], ctx->box[1], ctx->box[2]);
  p.bin_size = max_distance / (float)n_bins;
  p.inv_bin = 1.0f / p.bin_size;
  // squared lengths at or above this are past the last bin for sure
  const double cut = (double)max_distance * (1.0 + 1e-5);
  p.s2_cut = (float)(cut * cut);
  p.n_bins = n_bins;
  p.counts = (unsigned long long*)(base + o_cnt);
  if (n_q && l1.n > 0 && l2.n > 0) {
    const size_t shm = (size_t)8 * n_bins * 4;
    auto kern = symmetric ? pair_hist_kernel<true> : pair_hist_kernel<false>;
    if (shm > 48 * 1024)
      AMDAT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    AMDAT_REQUIRE(n_q <= 65535, "at most 65535 frames or time pairs per call");
    dim3 grid((unsigned)ceil_div(l1.n, PH_I_PER_BLOCK), (unsigned)n_q);
    KernelTimer kt(ctx, "pair_hist_kernel");
    kern<<<grid, PH_THREADS, shm, ctx->stream>>>(p);
    check_launch("pair_hist_kernel");
    count_launch(ctx);
  }
  AMDAT_CUDA(cudaMemcpyAsync(counts, base + o_cnt, n_out * 8,
                             out_flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             ctx->stream));
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_rdf_run(amdat_ctx* ctx, int32_t list1, int32_t list2, const int32_t* frames,
                           int32_t n_frames, float max_distance, int32_t n_bins, int32_t out_flags,
                           int64_t* counts) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    AMDAT_REQUIRE(frames != nullptr && n_frames >= 1, "need >= 1 frame");
    for (int f = 0; f < n_frames; ++f)
      AMDAT_REQUIRE(frames[f] >= 0 && frames[f] < ctx->n_frames, "frame index out of range");
    const ListEntry& a = list_entry(ctx, list1);
    const ListEntry& b = list_entry(ctx, list2);
    std::vector<int32_t> fa(frames, frames + n_frames), row(n_frames);
    for (int f = 0; f < n_frames; ++f) row[f] = f;
    run_pair_hist(ctx, a, b, list1 == list2, fa, fa, row, n_frames, max_distance, n_bins,
                  out_flags, counts);
  });
}

amdat_status amdat_vhd_run(amdat_ctx* ctx, int32_t list1, int32_t list2, int32_t fullblock,
                           float max_distance, int32_t n_bins, int32_t out_flags, int64_t* counts) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    const ListEntry& a = list_entry(ctx, list1);
    const ListEntry& b = list_entry(ctx, list2);
    const PairTable& P = pair_table(ctx, fullblock != 0, false);
    Pairs hp = scheme_pairs(ctx->scheme, fullblock != 0, false);
    // time pairs with t0 == t1 (gap 0) are the same-time pair loop: symmetric counting
    // applies only when t0 == t1; keep the general ordered loop for every pair.
    run_pair_hist(ctx, a, b, false, hp.t0, hp.t1, hp.gap, P.n_gaps, max_distance, n_bins,
                  out_flags, counts);
  });
}

}  // extern "C"
