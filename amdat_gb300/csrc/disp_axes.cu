// Per-axis displacement sums and the distribution of |dr|^2, the per-atom
// kernels of
//   Mean_Square_Displacement_2D::listkernel (src/mean_square_displacement_2d.cpp:143-146)
//   Mean_Displacement::listkernel           (src/mean_displacement.cpp:163-166)
//   DebyeWaller_Dist::listkernel            (src/debyewaller_dist.cpp:64-78)
//   Displacement_Distribution::listkernel   (src/displacement_distribution.cpp:69-83)
// over the time pairs of the scheduler: every gap (System::displacement_list,
// src/system.cpp:4090) or one gap (the single-gap variant, src/system.cpp:4349-4412,
// which visits exactly that gap's pairs of the full enumeration).
//
// Work items are (time pair, chunk of list members); a persistent grid pulls
// them from an atomic counter.  Per item a block accumulates, with
// Kahan-compensated FP32 per thread and compensated warp shuffles, the sums of
// dx, dy, dz, dx^2, dy^2, dz^2 and |dr|^4, writes one FP64 partial each, and
// adds its |dr|^2 histogram (shared memory, integer atomics) to the gap's
// counts.  A finalize kernel sums each gap's partials in item order (FP64).
//
// The histogram bin follows the reference's FP32 chain:
//   d = sqrtf((dx*dx + dy*dy) + dz*dz), u2 = float(pow(d, 2.0)) = float(double(d)^2),
//   bin = int(u2 / bin_size), clamped to the top bin (the overflow bin).
#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.h"

namespace amdat {

constexpr int AX_THREADS = 256;
constexpr int AX_CHUNK = 4096;
constexpr int AX_OUT = 7;  // dx, dy, dz, dx^2, dy^2, dz^2, |dr|^4

struct AxItem {
  int32_t pair, a0, a1, gap;
};

struct AxKSum {
  float s, c;
};
__device__ __forceinline__ void ax_add(AxKSum& k, float v) {
  const float y = __fsub_rn(v, k.c), t = __fadd_rn(k.s, y);
  k.c = __fsub_rn(__fsub_rn(t, k.s), y);
  k.s = t;
}

__global__ void __launch_bounds__(AX_THREADS)
    disp_axes_kernel(const float* __restrict__ u, int64_t n_pad, int32_t list_n, int32_t list_first,
                     const int32_t* __restrict__ list_idx, const int32_t* __restrict__ t0,
                     const int32_t* __restrict__ t1, const AxItem* __restrict__ items, int32_t n_items,
                     int32_t* __restrict__ counter, double* __restrict__ part, int32_t n_bins,
                     float bin_size, unsigned long long* __restrict__ counts) {
  extern __shared__ unsigned int hist[];  // [n_bins]
  __shared__ int s_item;
  __shared__ double s_red[AX_THREADS / 32][AX_OUT];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  (void)list_n;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const AxItem it = items[item];
    const float* X0 = u + (int64_t)t0[it.pair] * 3 * n_pad;
    const float* X1 = u + (int64_t)t1[it.pair] * 3 * n_pad;
    for (int b = tid; b < n_bins; b += AX_THREADS) hist[b] = 0u;
    __syncthreads();
    AxKSum acc[AX_OUT];
#pragma unroll
    for (int k = 0; k < AX_OUT; ++k) acc[k] = AxKSum{0.f, 0.f};
    for (int a = it.a0 + tid; a < it.a1; a += AX_THREADS) {
      const int atom = list_idx ? __ldg(list_idx + a) : list_first + a;
      const float dx = __fsub_rn(__ldg(X1 + atom), __ldg(X0 + atom));
      const float dy = __fsub_rn(__ldg(X1 + n_pad + atom), __ldg(X0 + n_pad + atom));
      const float dz = __fsub_rn(__ldg(X1 + 2 * n_pad + atom), __ldg(X0 + 2 * n_pad + atom));
      const float xx = __fmul_rn(dx, dx), yy = __fmul_rn(dy, dy), zz = __fmul_rn(dz, dz);
      ax_add(acc[0], dx);
      ax_add(acc[1], dy);
      ax_add(acc[2], dz);
      ax_add(acc[3], xx);
      ax_add(acc[4], yy);
      ax_add(acc[5], zz);
      const float d2 = __fadd_rn(__fadd_rn(xx, yy), zz);
      ax_add(acc[6], __fmul_rn(d2, d2));
      if (n_bins > 0) {
        const float d = __fsqrt_rn(d2);
        const float u2 = __double2float_rn((double)d * (double)d);
        int b = (int)__fdiv_rn(u2, bin_size);
        if (b >= n_bins || b < 0) b = n_bins - 1;  // top bin collects the overflow
        atomicAdd(hist + b, 1u);
      }
    }
    // compensated values -> per-warp FP64 sums -> one partial per output
#pragma unroll
    for (int k = 0; k < AX_OUT; ++k) {
      double v = (double)acc[k].s - (double)acc[k].c;
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (lane == 0) s_red[warp][k] = v;
    }
    __syncthreads();
    if (tid < AX_OUT) {
      double t = 0.0;
      for (int w = 0; w < AX_THREADS / 32; ++w) t += s_red[w][tid];
      part[(int64_t)item * AX_OUT + tid] = t;
    }
    if (n_bins > 0)
      for (int b = tid; b < n_bins; b += AX_THREADS)
        if (hist[b]) atomicAdd(counts + (int64_t)it.gap * n_bins + b, (unsigned long long)hist[b]);
    __syncthreads();
  }
}

// per gap: the item partials in item order (FP64)
__global__ void disp_axes_finalize_kernel(const double* __restrict__ part,
                                          const int32_t* __restrict__ gap_item, int32_t n_gaps,
                                          double* __restrict__ axis_sums, double* __restrict__ d4) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gaps) return;
  double s[AX_OUT] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = gap_item[g]; i < gap_item[g + 1]; ++i)
    for (int k = 0; k < AX_OUT; ++k) s[k] += part[(int64_t)i * AX_OUT + k];
  for (int k = 0; k < 6; ++k) axis_sums[(int64_t)g * 6 + k] = s[k];
  d4[g] = s[6];
}

}  // namespace amdat

using namespace amdat;

extern "C" amdat_status amdat_disp_axes_run(amdat_ctx* ctx, int32_t list, int32_t fullblock, int32_t gap,
                                            int32_t n_bins, float bin_size, int32_t out_flags,
                                            double* axis_sums, double* sum_d4, int64_t* atom_pairs,
                                            int64_t* d2_counts) {
  return guarded([&] {
    check_ctx(ctx);
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "no trajectory uploaded");
    if (!ctx->have_scheme) throw Error(AMDAT_ERR_STATE, "no time scheme set");
    AMDAT_REQUIRE(out_flags == AMDAT_OUT_HOST || out_flags == AMDAT_OUT_DEVICE, "bad out_flags");
    AMDAT_REQUIRE(n_bins >= 0 && n_bins <= 16384, "n_bins must be in [0, 16384]");
    AMDAT_REQUIRE(n_bins == 0 || bin_size > 0.0f, "bin_size must be positive");
    const ListEntry& e = list_entry(ctx, list);
    const PairTable& P = pair_table(ctx, fullblock != 0, false);
    const int G = P.n_gaps;
    AMDAT_REQUIRE(gap >= -1 && gap < G, "gap out of range");
    const int g0 = gap < 0 ? 0 : gap, g1 = gap < 0 ? G : gap + 1;
    // items: gap-major, (pair, member chunk)
    const int nch = (int)std::max<int64_t>(1, ceil_div(e.n, AX_CHUNK));
    std::vector<AxItem> items;
    std::vector<int32_t> gap_item(G + 1, 0);
    for (int g = 0; g < G; ++g) {
      gap_item[g] = (int32_t)items.size();
      if (g < g0 || g >= g1 || e.n == 0) continue;
      for (int p = P.gap_first[g]; p < P.gap_first[g + 1]; ++p)
        for (int c = 0; c < nch; ++c)
          items.push_back(AxItem{p, (int32_t)((int64_t)e.n * c / nch), (int32_t)((int64_t)e.n * (c + 1) / nch), g});
    }
    gap_item[G] = (int32_t)items.size();
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t o = 0;
    const size_t o_items = o; o = align(o + std::max<size_t>(items.size(), 1) * sizeof(AxItem));
    const size_t o_gi = o; o = align(o + gap_item.size() * 4);
    const size_t o_cnt = o; o = align(o + 4);
    const size_t o_part = o; o = align(o + std::max<size_t>(items.size(), 1) * AX_OUT * 8);
    const size_t o_ax = o; o = align(o + (size_t)G * 6 * 8);
    const size_t o_d4 = o; o = align(o + (size_t)G * 8);
    const size_t o_h = o; o = align(o + (size_t)G * std::max(n_bins, 1) * 8);
    unsigned char* base = ctx->scratch.reserve(o);
    cudaStream_t st = ctx->stream;
    if (!items.empty())
      AMDAT_CUDA(cudaMemcpyAsync(base + o_items, items.data(), items.size() * sizeof(AxItem), cudaMemcpyHostToDevice, st));
    AMDAT_CUDA(cudaMemcpyAsync(base + o_gi, gap_item.data(), gap_item.size() * 4, cudaMemcpyHostToDevice, st));
    AMDAT_CUDA(cudaMemsetAsync(base + o_cnt, 0, 4, st));
    AMDAT_CUDA(cudaMemsetAsync(base + o_ax, 0, o - o_ax, st));
    if (!items.empty()) {
      const size_t shm = (size_t)n_bins * 4;
      if (shm > 32 * 1024)
        AMDAT_CUDA(cudaFuncSetAttribute(disp_axes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
      const int grid = (int)std::min<int64_t>((int64_t)ctx->n_sm * 8, (int64_t)items.size());
      KernelTimer kt(ctx, "disp_axes_kernel");
      disp_axes_kernel<<<grid, AX_THREADS, shm, st>>>(
          ctx->u.ptr, ctx->n_pad, e.n, e.first, e.contiguous ? nullptr : e.idx.ptr, P.t0.ptr, P.t1.ptr,
          (const AxItem*)(base + o_items), (int32_t)items.size(), (int32_t*)(base + o_cnt),
          (double*)(base + o_part), n_bins, n_bins ? bin_size : 1.0f, (unsigned long long*)(base + o_h));
      check_launch("disp_axes_kernel");
      count_launch(ctx);
    }
    disp_axes_finalize_kernel<<<(unsigned)ceil_div(G, 128), 128, 0, st>>>(
        (const double*)(base + o_part), (const int32_t*)(base + o_gi), G, (double*)(base + o_ax),
        (double*)(base + o_d4));
    check_launch("disp_axes_finalize_kernel");
    count_launch(ctx);
    const cudaMemcpyKind kind = out_flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (axis_sums) AMDAT_CUDA(cudaMemcpyAsync(axis_sums, base + o_ax, (size_t)G * 6 * 8, kind, st));
    if (sum_d4) AMDAT_CUDA(cudaMemcpyAsync(sum_d4, base + o_d4, (size_t)G * 8, kind, st));
    if (d2_counts && n_bins) AMDAT_CUDA(cudaMemcpyAsync(d2_counts, base + o_h, (size_t)G * n_bins * 8, kind, st));
    if (atom_pairs) {
      std::vector<int64_t> c(G, 0);
      for (int g = g0; g < g1; ++g) c[g] = (int64_t)e.n * (P.gap_first[g + 1] - P.gap_first[g]);
      if (out_flags == AMDAT_OUT_DEVICE)
        AMDAT_CUDA(cudaMemcpyAsync(atom_pairs, c.data(), (size_t)G * 8, cudaMemcpyHostToDevice, st));
      else
        std::memcpy(atom_pairs, c.data(), (size_t)G * 8);
      AMDAT_CUDA(cudaStreamSynchronize(st));
    }
    AMDAT_CUDA(cudaStreamSynchronize(st));
  });
}
