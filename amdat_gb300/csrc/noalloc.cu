// Displacement moments without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need a
// mean-square displacement: code running inside a memory pool or arena that
// owns all of the GPU's memory, plugin hosts that forbid cudaMalloc after
// start-up, or callers that must not trigger allocation-related
// synchronisation.  amdat_disp_moments_noalloc serves them.  The caller passes
// its own device input (unwrapped coordinates) and device outputs.  Every
// temporary the run needs (time-pair table, work items, per-item partial sums,
// the work counter) lives in one file-scope __device__ array of
// NOALLOC_SCRATCH_BYTES, which the driver places in device memory when the
// library's module is loaded: every GPU that loads this library holds those
// bytes until the process exits, used or not.
//
// The host finds the array's device address with cudaGetSymbolAddress once per
// device (the first call on each device, with that device current), then
// passes it to the kernels.  Each call copies its tables from host vectors it
// frees on return, so a stream under capture is refused (AMDAT_ERR_STATE).
// All calls share the one array and it keeps the last call's contents: each
// call clears the work counter itself, and two calls whose GPU work overlaps
// (different streams, or host threads on the same device) race on the array,
// so callers must order them.
#include <cstring>
#include <mutex>
#include <vector>

#include "engine.h"

namespace amdat {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)16 << 20;  // 16 MiB
constexpr int NOALLOC_MAX_DEVICES = 64;
constexpr int NOALLOC_THREADS = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocItem {
  int32_t pair, a0, a1, pad;
};

// one block per item: sum |dr|^2 and |dr|^4 over atoms a0..a1 of one time pair,
// read straight from the caller's [frame][atom][3] array, compensated FP32
__global__ void __launch_bounds__(NOALLOC_THREADS)
    noalloc_moments_kernel(const float* __restrict__ xyz, int32_t n_atoms,
                           const int32_t* __restrict__ t0, const int32_t* __restrict__ t1,
                           const NoallocItem* __restrict__ items, int32_t n_items,
                           int32_t* __restrict__ counter, double* __restrict__ part) {
  __shared__ int s_item;
  __shared__ float s_red[NOALLOC_THREADS / 32][4];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const NoallocItem it = items[item];
    const float* A = xyz + (int64_t)t0[it.pair] * n_atoms * 3;
    const float* B = xyz + (int64_t)t1[it.pair] * n_atoms * 3;
    float s2 = 0.f, c2 = 0.f, s4 = 0.f, c4 = 0.f;
    for (int a = it.a0 + threadIdx.x; a < it.a1; a += blockDim.x) {
      const float dx = __fsub_rn(__ldg(B + 3 * a), __ldg(A + 3 * a));
      const float dy = __fsub_rn(__ldg(B + 3 * a + 1), __ldg(A + 3 * a + 1));
      const float dz = __fsub_rn(__ldg(B + 3 * a + 2), __ldg(A + 3 * a + 2));
      const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      float y = __fsub_rn(d2, c2), t = __fadd_rn(s2, y);
      c2 = __fsub_rn(__fsub_rn(t, s2), y);
      s2 = t;
      y = __fsub_rn(d2 * d2, c4);
      t = __fadd_rn(s4, y);
      c4 = __fsub_rn(__fsub_rn(t, s4), y);
      s4 = t;
    }
    // per-warp sums of the compensated values, then FP64 across warps
    float v[4] = {s2, -c2, s4, -c4};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
    if ((threadIdx.x & 31) == 0)
      for (int k = 0; k < 4; ++k) s_red[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 2) {
      double acc = 0.0;
      for (int w = 0; w < NOALLOC_THREADS / 32; ++w)
        acc += (double)s_red[w][2 * threadIdx.x] + (double)s_red[w][2 * threadIdx.x + 1];
      part[2 * (int64_t)item + threadIdx.x] = acc;
    }
    __syncthreads();
  }
}

// sums the partials of each gap in item order (FP64) into the caller's outputs
__global__ void noalloc_finalize_kernel(const double* __restrict__ part,
                                        const int32_t* __restrict__ gap_item_first, int32_t n_gaps,
                                        double* __restrict__ d2, double* __restrict__ d4) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gaps) return;
  double a = 0.0, b = 0.0;
  for (int i = gap_item_first[g]; i < gap_item_first[g + 1]; ++i) {
    a += part[2 * (int64_t)i];
    b += part[2 * (int64_t)i + 1];
  }
  d2[g] = a;
  d4[g] = b;
}

static unsigned char* noalloc_scratch_address() {
  static std::mutex mu;
  static unsigned char* addr[NOALLOC_MAX_DEVICES] = {nullptr};
  int dev = 0;
  AMDAT_CUDA(cudaGetDevice(&dev));
  AMDAT_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES, "device index beyond the supported range");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    // the host-side name g_noalloc_scratch is not a device address: ask the runtime
    AMDAT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[dev] = (unsigned char*)p;
  }
  return addr[dev];
}

}  // namespace amdat

using namespace amdat;

extern "C" amdat_status amdat_disp_moments_noalloc(const amdat_scheme* scheme, int32_t fullblock,
                                                   const float* d_xyz, int32_t n_frames,
                                                   int32_t n_atoms, void* cuda_stream,
                                                   double* d_sum_d2, double* d_sum_d4) {
  return guarded([&] {
    AMDAT_REQUIRE(scheme != nullptr && d_xyz != nullptr && d_sum_d2 != nullptr && d_sum_d4 != nullptr,
                  "null argument");
    AMDAT_REQUIRE(n_frames >= 1 && n_atoms >= 1, "need >= 1 frame and >= 1 atom");
    scheme_check(*scheme);
    const Pairs P = scheme_pairs(*scheme, fullblock != 0, false);
    const int G = scheme_n_timegaps(*scheme);
    for (size_t i = 0; i < P.t1.size(); ++i)
      AMDAT_REQUIRE(P.t1[i] < n_frames, "time scheme needs more frames than the coordinates hold");
    // work items: (pair, atom chunk), gap-major so each gap's items are contiguous
    const int64_t n_pairs = (int64_t)P.gap.size();
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t fixed = align(sizeof(int32_t)) + 2 * align(n_pairs * sizeof(int32_t)) +
                         align((G + 1) * sizeof(int32_t));
    AMDAT_REQUIRE(fixed < NOALLOC_SCRATCH_BYTES / 2,
                  "time scheme too large for the 16 MiB no-allocation scratch");
    const int64_t max_items = (int64_t)((NOALLOC_SCRATCH_BYTES - fixed - 1024) /
                                        (sizeof(NoallocItem) + 2 * sizeof(double)));
    // every time pair needs at least one item (one chunk of all atoms): a scheme
    // with more pairs than items cannot run here, whatever the chunk size
    if (n_pairs > max_items)
      throw Error(AMDAT_ERR_ARGUMENT,
                  "time scheme has " + std::to_string(n_pairs) + " time pairs; the 16 MiB "
                  "no-allocation scratch holds at most " + std::to_string(max_items) +
                  " for this scheme");
    // chunks of 4096 atoms, doubled until the items fit; at most one chunk per pair
    int64_t chunk = 4096;
    while (chunk < n_atoms && n_pairs * ceil_div(n_atoms, chunk) > max_items) chunk *= 2;
    const int nch = (int)ceil_div(n_atoms, chunk);
    std::vector<NoallocItem> items;
    items.reserve((size_t)(n_pairs * nch));
    std::vector<int32_t> gap_first(G + 1, 0);
    for (int g = 0; g < G; ++g) {
      gap_first[g] = (int32_t)items.size();
      for (int p = P.gap_first[g]; p < P.gap_first[g + 1]; ++p)
        for (int c = 0; c < nch; ++c)
          items.push_back(NoallocItem{p, (int32_t)((int64_t)n_atoms * c / nch),
                                      (int32_t)((int64_t)n_atoms * (c + 1) / nch), 0});
    }
    gap_first[G] = (int32_t)items.size();
    // the table copies below read host vectors freed on return: a captured
    // graph would keep their addresses, so capture is refused
    cudaStream_t st = (cudaStream_t)cuda_stream;
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing(st, &capture);
    if (ce == cudaErrorStreamCaptureImplicit || (ce == cudaSuccess && capture != cudaStreamCaptureStatusNone)) {
      (void)cudaGetLastError();
      throw Error(AMDAT_ERR_STATE, "amdat_disp_moments_noalloc cannot run on a stream under capture");
    }
    AMDAT_CUDA(ce);
    // scratch layout: [counter | t0 | t1 | gap_first | items | partials]
    unsigned char* base = noalloc_scratch_address();
    size_t o = 0;
    const size_t o_counter = o; o = align(o + sizeof(int32_t));
    const size_t o_t0 = o; o = align(o + n_pairs * sizeof(int32_t));
    const size_t o_t1 = o; o = align(o + n_pairs * sizeof(int32_t));
    const size_t o_gf = o; o = align(o + (G + 1) * sizeof(int32_t));
    const size_t o_items = o; o = align(o + items.size() * sizeof(NoallocItem));
    const size_t o_part = o; o = align(o + items.size() * 2 * sizeof(double));
    AMDAT_REQUIRE(o <= NOALLOC_SCRATCH_BYTES, "work exceeds the 16 MiB no-allocation scratch");
    AMDAT_CUDA(cudaMemsetAsync(base + o_counter, 0, sizeof(int32_t), st));
    if (n_pairs) {
      AMDAT_CUDA(cudaMemcpyAsync(base + o_t0, P.t0.data(), n_pairs * 4, cudaMemcpyHostToDevice, st));
      AMDAT_CUDA(cudaMemcpyAsync(base + o_t1, P.t1.data(), n_pairs * 4, cudaMemcpyHostToDevice, st));
    }
    AMDAT_CUDA(cudaMemcpyAsync(base + o_gf, gap_first.data(), (G + 1) * 4, cudaMemcpyHostToDevice, st));
    if (!items.empty())
      AMDAT_CUDA(cudaMemcpyAsync(base + o_items, items.data(), items.size() * sizeof(NoallocItem),
                                 cudaMemcpyHostToDevice, st));
    if (!items.empty()) {
      int dev = 0, n_sm = 0;
      AMDAT_CUDA(cudaGetDevice(&dev));
      AMDAT_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
      const int grid = (int)std::min<int64_t>((int64_t)n_sm * 8, (int64_t)items.size());
      noalloc_moments_kernel<<<grid, NOALLOC_THREADS, 0, st>>>(
          d_xyz, n_atoms, (const int32_t*)(base + o_t0), (const int32_t*)(base + o_t1),
          (const NoallocItem*)(base + o_items), (int32_t)items.size(), (int32_t*)(base + o_counter),
          (double*)(base + o_part));
      check_launch("noalloc_moments_kernel");
    }
    noalloc_finalize_kernel<<<(unsigned)ceil_div(G, 128), 128, 0, st>>>(
        (const double*)(base + o_part), (const int32_t*)(base + o_gf), G, d_sum_d2, d_sum_d4);
    check_launch("noalloc_finalize_kernel");
    // the host tables above are pageable: copies from them complete before the
    // calls return, so nothing outlives this function
  });
}
