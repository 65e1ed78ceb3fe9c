// Coherent intermediate scattering function and static structure factor from
// Fourier-density tables.
//
// Replaces Intermediate_Scattering_Function::displacementkernel
// (src/intermediate_scattering_function.cpp:551-566): for every time pair
// (t0, t1) that System::displacement_loop visits (src/system.cpp:3918-3964),
// corr[g][shell] += sum_{k in shell} Re(rho1(k,t0) conj(rho2(k,t1))) / H_shell,
// and Structure_Factor::timekernel (src/structure_factor.cpp:201-230):
// S[shell] += sum_{k in shell} |rho(k,t)|^2 / H_shell per frame.
//
// The k axis is cut into shell-aligned tiles of up to 32 vectors.  A block
// stages its tile's density for every frame in shared memory (T x 32 x 8 B),
// then each warp owns a residue class of gaps: for each of its gaps a lane
// (one k) runs over the gap's time pairs with a Kahan-compensated FP32 sum of
// products, and the warp folds its 32 vectors with shuffles into one FP64
// partial per (tile, gap).  A finalize kernel adds the partials of each
// (shell, gap) in tile order in FP64 and divides by the shell size, so the
// result is deterministic.  Linear schemes (lagged pair tables) take
// isf_lag_kernel, which reuses each frame's density across 8 gaps.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "engine.h"

namespace amdat {

struct KTile {
  int32_t k0, nk, shell;
};

struct KSumF {
  float s, c;
};
__device__ __forceinline__ void ksadd(KSumF& k, float v) {
  float y = __fsub_rn(v, k.c), t = __fadd_rn(k.s, y);
  k.c = __fsub_rn(__fsub_rn(t, k.s), y);
  k.s = t;
}

template <int KT>
__global__ void __launch_bounds__(256)
    isf_pairs_kernel(const float2* __restrict__ rho1, const float2* __restrict__ rho2,
                     int32_t n_frames, int32_t n_k, const KTile* __restrict__ tiles,
                     const int32_t* __restrict__ t0, const int32_t* __restrict__ t1,
                     const int32_t* __restrict__ gap_first, int32_t n_gaps,
                     double* __restrict__ part) {
  extern __shared__ float2 sh[];
  const bool same = rho1 == rho2;
  float2* s1 = sh;
  float2* s2 = same ? sh : sh + (size_t)n_frames * KT;
  const KTile T = tiles[blockIdx.x];
  for (int i = threadIdx.x; i < n_frames * KT; i += blockDim.x) {
    const int f = i / KT, k = i % KT;
    const float2 z = make_float2(0.f, 0.f);
    s1[i] = k < T.nk ? rho1[(int64_t)f * n_k + T.k0 + k] : z;
    if (!same) s2[i] = k < T.nk ? rho2[(int64_t)f * n_k + T.k0 + k] : z;
  }
  __syncthreads();
  const int kk = threadIdx.x % KT;
  const int grp = threadIdx.x / KT, n_grp = blockDim.x / KT;
  // the loop bound is uniform across the block, so every lane of a warp
  // reaches each shuffle together even when several groups share a warp
  for (int gb = 0; gb < n_gaps; gb += n_grp) {
    const int g = gb + grp;
    KSumF acc = {0.f, 0.f};
    if (g < n_gaps) {
      for (int p = gap_first[g]; p < gap_first[g + 1]; ++p) {
        const float2 a = s1[t0[p] * KT + kk], b = s2[t1[p] * KT + kk];
        ksadd(acc, fmaf(a.x, b.x, a.y * b.y));
      }
    }
    double v = (double)acc.s - (double)acc.c;
#pragma unroll
    for (int off = KT / 2; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off, KT);
    if (kk == 0 && g < n_gaps) part[(int64_t)blockIdx.x * n_gaps + g] = v;
  }
}

// Lagged pair tables (the linear schemes: gap g's pairs are (t, t + lag_g) for
// t = 0 .. cnt_g - 1): a warp owns blocks of 8 gaps with consecutive lags and a
// lane (one k) runs once over t.  rho1(t) is read once per step, and
// rho2(t + lag) of the 8 gaps sits in a register window that slides by one
// frame per step (one new load), so two shared-memory loads feed 8 products.
// Each gap keeps its Kahan sum in t order, the pair order of the table, so the
// partials equal the pair-table kernel's.
__global__ void __launch_bounds__(256)
    isf_lag_kernel(const float2* __restrict__ rho1, const float2* __restrict__ rho2, int32_t n_frames,
                   int32_t n_k, const KTile* __restrict__ tiles, const int32_t* __restrict__ lag,
                   const int32_t* __restrict__ gap_first, int32_t n_gaps, double* __restrict__ part) {
  constexpr int KT = 32;
  extern __shared__ float2 sh[];
  const bool same = rho1 == rho2;
  float2* s1 = sh;
  float2* s2 = same ? sh : sh + (size_t)n_frames * KT;
  const KTile T = tiles[blockIdx.x];
  for (int i = threadIdx.x; i < n_frames * KT; i += blockDim.x) {
    const int f = i / KT, k = i % KT;
    const float2 z = make_float2(0.f, 0.f);
    s1[i] = k < T.nk ? rho1[(int64_t)f * n_k + T.k0 + k] : z;
    if (!same) s2[i] = k < T.nk ? rho2[(int64_t)f * n_k + T.k0 + k] : z;
  }
  __syncthreads();
  const int kk = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  const float2 zero = make_float2(0.f, 0.f);
  for (int g0 = 8 * warp; g0 < n_gaps; g0 += 8 * n_warps) {
    int cnt[8], tmax = 0;
    bool window = true;  // lags g0 .. g0+7 consecutive (gaps without pairs do not matter)
    const int lag0 = lag[g0];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      cnt[j] = g0 + j < n_gaps ? gap_first[g0 + j + 1] - gap_first[g0 + j] : 0;
      if (cnt[j] > 0 && lag[g0 + j] != lag0 + j) window = false;
      tmax = max(tmax, cnt[j]);
    }
    KSumF acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = KSumF{0.f, 0.f};
    if (window) {
      // r[(u + j) & 7] holds rho2(t + lag0 + j) at step u of each 8-step round
      float2 r[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) r[j] = lag0 + j < n_frames ? s2[(lag0 + j) * KT + kk] : zero;
      for (int t0 = 0; t0 < tmax; t0 += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int t = t0 + u;
          if (t < tmax) {
            const float2 a = s1[t * KT + kk];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const float2 b = r[(u + j) & 7];
              if (t < cnt[j]) ksadd(acc[j], fmaf(a.x, b.x, a.y * b.y));
            }
            const int tn = t + 1 + lag0 + 7;
            r[u & 7] = tn < n_frames ? s2[tn * KT + kk] : zero;
          }
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (cnt[j] == 0) continue;
        const int L = lag[g0 + j];
        for (int t = 0; t < cnt[j]; ++t) {
          const float2 a = s1[t * KT + kk], b = s2[(t + L) * KT + kk];
          ksadd(acc[j], fmaf(a.x, b.x, a.y * b.y));
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      double v = (double)acc[j].s - (double)acc[j].c;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (kk == 0 && g0 + j < n_gaps) part[(int64_t)blockIdx.x * n_gaps + g0 + j] = v;
    }
  }
}

__global__ void tile_finalize_kernel(const double* __restrict__ part, int32_t n_cols,
                                     const int32_t* __restrict__ shell_tile_first,
                                     const float* __restrict__ inv_count, int32_t n_shells,
                                     double* __restrict__ out /* [col][shell] */) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)n_shells * n_cols) return;
  const int s = (int)(i % n_shells), col = (int)(i / n_shells);
  double acc = 0.0;
  for (int t = shell_tile_first[s]; t < shell_tile_first[s + 1]; ++t) acc += part[(int64_t)t * n_cols + col];
  out[(int64_t)col * n_shells + s] = acc * (double)inv_count[s];
}

__global__ void __launch_bounds__(256)
    sk_frames_kernel(const float2* __restrict__ rho1, const float2* __restrict__ rho2,
                     int32_t n_frames, int32_t n_k, const KTile* __restrict__ tiles,
                     double* __restrict__ part) {
  __shared__ double red[8];
  const KTile T = tiles[blockIdx.x];
  KSumF acc = {0.f, 0.f};
  if ((int)threadIdx.x < T.nk) {
    const int k = T.k0 + threadIdx.x;
    for (int f = 0; f < n_frames; ++f) {
      const float2 a = rho1[(int64_t)f * n_k + k], b = rho2[(int64_t)f * n_k + k];
      ksadd(acc, fmaf(a.x, b.x, a.y * b.y));
    }
  }
  double v = (double)acc.s - (double)acc.c;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

static void make_tiles(const int32_t* off, int32_t n_shells, int32_t width, int32_t n_k,
                       std::vector<KTile>& tiles, std::vector<int32_t>& shell_tile_first,
                       std::vector<float>& inv_count) {
  AMDAT_REQUIRE(off != nullptr && n_shells >= 1, "need >= 1 shell");
  AMDAT_REQUIRE(off[0] >= 0 && off[n_shells] <= n_k, "shell offsets outside the density's vectors");
  tiles.clear();
  shell_tile_first.assign(n_shells + 1, 0);
  inv_count.assign(n_shells, 0.f);
  for (int s = 0; s < n_shells; ++s) {
    AMDAT_REQUIRE(off[s + 1] >= off[s], "shell offsets must ascend");
    shell_tile_first[s] = (int32_t)tiles.size();
    for (int k = off[s]; k < off[s + 1]; k += width)
      tiles.push_back(KTile{k, std::min(width, off[s + 1] - k), s});
    const int cnt = off[s + 1] - off[s];
    inv_count[s] = cnt ? 1.0f / (float)cnt : 0.0f;
  }
  shell_tile_first[n_shells] = (int32_t)tiles.size();
}

template <class T>
static void out_copy(amdat_ctx* ctx, T* dst, const T* src, size_t n, int32_t flags) {
  if (!dst || !n) return;
  AMDAT_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T),
                             flags == AMDAT_OUT_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             ctx->stream));
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_isf_run(amdat_ctx* ctx, int32_t h1, int32_t h2, int32_t fullblock,
                           const int32_t* shell_offsets, int32_t n_shells, int32_t out_flags,
                           double* corr_sum, int64_t* pair_count) {
  return guarded([&] {
    check_ctx(ctx);
    Density& d1 = density(ctx, h1);
    Density& d2 = density(ctx, h2);
    AMDAT_REQUIRE(d1.n_k == d2.n_k && d1.n_frames == d2.n_frames, "densities differ in shape");
    const int T = d1.n_frames;
    for (int f = 0; f < T; ++f)
      AMDAT_REQUIRE(d1.frames[f] == f && d2.frames[f] == f,
                    "coherent ISF needs densities over every frame 0..T-1");
    const PairTable& P = pair_table(ctx, fullblock != 0, true);
    AMDAT_REQUIRE(T >= scheme_n_timesteps(ctx->scheme),
                  "coherent ISF needs densities over every frame of the time scheme");
    const bool same = h1 == h2;
    int KT = 32;
    while (KT > 1 && (size_t)(same ? 1 : 2) * T * KT * sizeof(float2) > 200 * 1024) KT >>= 1;
    AMDAT_REQUIRE((size_t)(same ? 1 : 2) * T * KT * sizeof(float2) <= 200 * 1024,
                  "too many frames for the correlator's shared-memory tile");
    std::vector<KTile> tiles;
    std::vector<int32_t> stf;
    std::vector<float> invc;
    make_tiles(shell_offsets, n_shells, KT, d1.n_k, tiles, stf, invc);
    const int G = P.n_gaps;
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t o = 0;
    const size_t o_t = o; o = align(o + std::max<size_t>(tiles.size(), 1) * sizeof(KTile));
    const size_t o_gf = o; o = align(o + (G + 1) * 4);
    const size_t o_lag = o; o = align(o + std::max(G, 1) * 4);
    const size_t o_stf = o; o = align(o + stf.size() * 4);
    const size_t o_inv = o; o = align(o + invc.size() * 4);
    const size_t o_part = o; o = align(o + std::max<size_t>(tiles.size(), 1) * G * 8);
    const size_t o_out = o; o = align(o + (size_t)G * n_shells * 8);
    unsigned char* base = ctx->scratch.reserve(o);
    std::vector<unsigned char> host(o_part, 0);
    std::memcpy(host.data() + o_t, tiles.data(), tiles.size() * sizeof(KTile));
    std::memcpy(host.data() + o_gf, P.gap_first.data(), (G + 1) * 4);
    if (P.lagged) std::memcpy(host.data() + o_lag, P.lag.data(), G * 4);
    std::memcpy(host.data() + o_stf, stf.data(), stf.size() * 4);
    std::memcpy(host.data() + o_inv, invc.data(), invc.size() * 4);
    AMDAT_CUDA(cudaMemcpyAsync(base, host.data(), o_part, cudaMemcpyHostToDevice, ctx->stream));
    double* part = (double*)(base + o_part);
    double* out = (double*)(base + o_out);
    if (!tiles.empty()) {
      const size_t shm = (size_t)(same ? 1 : 2) * T * KT * sizeof(float2);
      auto launch = [&](auto kernel) {
        AMDAT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        KernelTimer kt(ctx, "isf_pairs_kernel");
        kernel<<<(unsigned)tiles.size(), 256, shm, ctx->stream>>>(
            d1.rho->ptr, d2.rho->ptr, T, d1.n_k, (const KTile*)(base + o_t), P.t0.ptr, P.t1.ptr,
            (const int32_t*)(base + o_gf), G, part);
      };
      const char* force = std::getenv("AMDAT_ISF_KERNEL");  // "pairs": the pair-table kernel always
      // linear schemes with enough gaps to occupy the block's 8 warps (8 gaps each)
      if (P.lagged && KT == 32 && G >= 64 && !(force && std::strcmp(force, "pairs") == 0)) {
        AMDAT_CUDA(cudaFuncSetAttribute(isf_lag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        KernelTimer kt(ctx, "isf_lag_kernel");
        isf_lag_kernel<<<(unsigned)tiles.size(), 256, shm, ctx->stream>>>(
            d1.rho->ptr, d2.rho->ptr, T, d1.n_k, (const KTile*)(base + o_t), (const int32_t*)(base + o_lag),
            (const int32_t*)(base + o_gf), G, part);
      } else switch (KT) {
        case 32: launch(isf_pairs_kernel<32>); break;
        case 16: launch(isf_pairs_kernel<16>); break;
        case 8: launch(isf_pairs_kernel<8>); break;
        case 4: launch(isf_pairs_kernel<4>); break;
        case 2: launch(isf_pairs_kernel<2>); break;
        default: launch(isf_pairs_kernel<1>); break;
      }
      check_launch("isf correlator kernel");
      count_launch(ctx);
    } else {
      AMDAT_CUDA(cudaMemsetAsync(part, 0, G * 8, ctx->stream));
    }
    const int64_t n_out = (int64_t)G * n_shells;
    tile_finalize_kernel<<<(unsigned)ceil_div(n_out, 256), 256, 0, ctx->stream>>>(
        part, G, (const int32_t*)(base + o_stf), (const float*)(base + o_inv), n_shells, out);
    check_launch("tile_finalize_kernel");
    count_launch(ctx);
    out_copy(ctx, corr_sum, out, (size_t)n_out, out_flags);
    if (pair_count) {
      std::vector<int64_t> pc(G);
      for (int g = 0; g < G; ++g) pc[g] = P.gap_first[g + 1] - P.gap_first[g];
      if (out_flags == AMDAT_OUT_DEVICE)
        AMDAT_CUDA(cudaMemcpyAsync(pair_count, pc.data(), G * 8, cudaMemcpyHostToDevice, ctx->stream));
      else
        std::memcpy(pair_count, pc.data(), G * 8);
    }
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

amdat_status amdat_structure_factor_run(amdat_ctx* ctx, int32_t h1, int32_t h2,
                                        const int32_t* shell_offsets, int32_t n_shells,
                                        int32_t out_flags, double* s_sum) {
  return guarded([&] {
    check_ctx(ctx);
    Density& d1 = density(ctx, h1);
    Density& d2 = density(ctx, h2);
    AMDAT_REQUIRE(d1.n_k == d2.n_k && d1.n_frames == d2.n_frames, "densities differ in shape");
    std::vector<KTile> tiles;
    std::vector<int32_t> stf;
    std::vector<float> invc;
    make_tiles(shell_offsets, n_shells, 256, d1.n_k, tiles, stf, invc);
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t o = 0;
    const size_t o_t = o; o = align(o + std::max<size_t>(tiles.size(), 1) * sizeof(KTile));
    const size_t o_stf = o; o = align(o + stf.size() * 4);
    const size_t o_inv = o; o = align(o + invc.size() * 4);
    const size_t o_part = o; o = align(o + std::max<size_t>(tiles.size(), 1) * 8);
    const size_t o_out = o; o = align(o + (size_t)n_shells * 8);
    unsigned char* base = ctx->scratch.reserve(o);
    std::vector<unsigned char> host(o_part, 0);
    std::memcpy(host.data() + o_t, tiles.data(), tiles.size() * sizeof(KTile));
    std::memcpy(host.data() + o_stf, stf.data(), stf.size() * 4);
    std::memcpy(host.data() + o_inv, invc.data(), invc.size() * 4);
    AMDAT_CUDA(cudaMemcpyAsync(base, host.data(), o_part, cudaMemcpyHostToDevice, ctx->stream));
    double* part = (double*)(base + o_part);
    double* out = (double*)(base + o_out);
    if (!tiles.empty()) {
      KernelTimer kt(ctx, "sk_frames_kernel");
      sk_frames_kernel<<<(unsigned)tiles.size(), 256, 0, ctx->stream>>>(
          d1.rho->ptr, d2.rho->ptr, d1.n_frames, d1.n_k, (const KTile*)(base + o_t), part);
      check_launch("sk_frames_kernel");
      count_launch(ctx);
    }
    tile_finalize_kernel<<<(unsigned)ceil_div(n_shells, 256), 256, 0, ctx->stream>>>(
        part, 1, (const int32_t*)(base + o_stf), (const float*)(base + o_inv), n_shells, out);
    check_launch("tile_finalize_kernel");
    count_launch(ctx);
    out_copy(ctx, s_sum, out, (size_t)n_shells, out_flags);
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

}  // extern "C"
