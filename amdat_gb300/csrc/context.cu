// Context, trajectory store and lists of the amdat_gb300 C ABI.
//
// The trajectory store replaces AMDAT's per-atom Coordinate arrays
// (src/trajectory.h:37-38: 'coordinates' wrapped, 'unwrapped') with frame-major
// FP32 structure-of-arrays planes in HBM: plane (t, c) holds coordinate c of
// every atom at frame t, padded to a multiple of 128 atoms so that every
// plane starts 512-byte aligned and vector (float4) loads stay aligned.
// Unwrapped coordinates are stored re-referenced to frame 0 (u(t) = r(t) -
// r(0)), so displacements r(t1)-r(t0) = u(t1)-u(t0) are formed from small
// numbers.  Wrapped coordinates are kept as read, or derived from unwrapped
// ones exactly as AMDAT's custom reader does (src/system.cpp read_custom,
// 'calc_wrapped': c = u - L*floor((u-lo)/L), every step in FP32).
#include <cstdio>
#include <cstring>

#include "engine.h"

namespace amdat {

static thread_local std::string g_last_error;
void set_last_error(const std::string& m) { g_last_error = m; }

void count_launch(amdat_ctx* ctx, int n) { ctx->launches += n; }

void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    throw Error(AMDAT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

amdat_ctx* check_ctx(amdat_ctx* ctx) {
  if (!ctx) throw Error(AMDAT_ERR_ARGUMENT, "null context");
  AMDAT_CUDA(cudaSetDevice(ctx->device));
  return ctx;
}

const ListEntry& list_entry(amdat_ctx* ctx, int32_t handle) {
  if (handle < 0 || handle >= (int32_t)ctx->lists.size())
    throw Error(AMDAT_ERR_ARGUMENT, "unknown list handle " + std::to_string(handle));
  return *ctx->lists[handle];
}

const PairTable& pair_table(amdat_ctx* ctx, bool fullblock, bool loop_order) {
  if (!ctx->have_scheme) throw Error(AMDAT_ERR_STATE, "no time scheme set (amdat_set_scheme)");
  const int key = (fullblock ? 2 : 0) + (loop_order ? 1 : 0);
  auto it = ctx->pair_cache.find(key);
  if (it != ctx->pair_cache.end()) return *it->second;
  Pairs p = scheme_pairs(ctx->scheme, fullblock, loop_order);
  for (size_t i = 0; i < p.t1.size(); ++i)
    if (p.t1[i] >= ctx->n_frames || p.t0[i] < 0)
      throw Error(AMDAT_ERR_STATE, "time scheme needs " + std::to_string(p.t1[i] + 1) +
                                       " frames, trajectory has " + std::to_string(ctx->n_frames));
  auto* t = new PairTable();
  t->n_pairs = (int64_t)p.gap.size();
  t->n_gaps = scheme_n_timegaps(ctx->scheme);
  t->gap_first = p.gap_first;
  t->lagged = true;
  t->lag.assign(t->n_gaps, 0);
  for (int g = 0; g < t->n_gaps && t->lagged; ++g)
    for (int i = p.gap_first[g]; i < p.gap_first[g + 1]; ++i) {
      const int k = i - p.gap_first[g];
      if (k == 0) t->lag[g] = p.t1[i] - p.t0[i];
      if (p.t0[i] != k || p.t1[i] - p.t0[i] != t->lag[g]) {
        t->lagged = false;
        break;
      }
    }
  const size_t n = p.gap.size();
  t->t0.reserve(n);
  t->t1.reserve(n);
  t->gap.reserve(n);
  t->h_t0 = p.t0;
  t->h_t1 = p.t1;
  t->h_gap = p.gap;
  AMDAT_CUDA(cudaMemcpy(t->t0.ptr, p.t0.data(), n * 4, cudaMemcpyHostToDevice));
  AMDAT_CUDA(cudaMemcpy(t->t1.ptr, p.t1.data(), n * 4, cudaMemcpyHostToDevice));
  AMDAT_CUDA(cudaMemcpy(t->gap.ptr, p.gap.data(), n * 4, cudaMemcpyHostToDevice));
  ctx->pair_cache[key] = t;
  return *t;
}

// ---------------------------------------------------------------------------
// staging kernels: host AoS [T][N][3] -> SoA planes [T][3][n_pad]
// ---------------------------------------------------------------------------

// FP32 ops with explicit rounding, no contraction: the wrapped coordinates
// must equal the reference's to the bit.
__device__ __forceinline__ float wrap_coord(float u, float lo, float L) {
  float f = floorf(__fdiv_rn(__fsub_rn(u, lo), L));
  return __fsub_rn(u, __fmul_rn(L, f));
}

template <class Real>
__global__ void stage_kernel(const Real* __restrict__ raw, const Real* __restrict__ raw_w,
                             int32_t T, int32_t N, int32_t n_pad, float3 box, float3 lo,
                             float* __restrict__ u, float* __restrict__ w) {
  const int64_t total = (int64_t)T * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t t = (int32_t)(i / N), a = (int32_t)(i % N);
    const Real* r = raw + i * 3;
    const Real* r0 = raw + (int64_t)a * 3;
    const float Ls[3] = {box.x, box.y, box.z}, los[3] = {lo.x, lo.y, lo.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t o = ((int64_t)t * 3 + c) * n_pad + a;
      // re-referenced displacement from frame 0, one rounding to FP32
      u[o] = (float)(r[c] - r0[c]);
      float wc;
      if (raw_w) {
        wc = (float)raw_w[i * 3 + c];
      } else {
        wc = wrap_coord((float)r[c], los[c], Ls[c]);
      }
      w[o] = wc;
    }
  }
}

template <class Real>
static void upload_impl(amdat_ctx* ctx, int32_t T, int32_t N, const Real* unwrapped,
                        const Real* wrapped, bool device_src, const float* box,
                        const float* box_lo) {
  AMDAT_REQUIRE(T >= 1 && N >= 1, "trajectory needs >= 1 frame and >= 1 atom");
  AMDAT_REQUIRE(unwrapped != nullptr && box != nullptr, "null trajectory or box");
  AMDAT_REQUIRE((int64_t)T * N < (int64_t)1 << 40, "trajectory too large");
  for (int c = 0; c < 3; ++c) AMDAT_REQUIRE(box[c] > 0.0f, "box lengths must be positive");
  const int32_t n_pad = (int32_t)ceil_div(N, 128) * 128;
  const size_t plane = (size_t)T * 3 * n_pad;
  ctx->have_traj = false;
  ctx->u.reserve(plane);
  ctx->w.reserve(plane);
  // padding atoms read as zeros (never part of a list)
  AMDAT_CUDA(cudaMemsetAsync(ctx->u.ptr, 0, plane * sizeof(float), ctx->stream));
  AMDAT_CUDA(cudaMemsetAsync(ctx->w.ptr, 0, plane * sizeof(float), ctx->stream));
  ctx->u64.release();
  ctx->w64.release();
  const size_t raw_bytes = (size_t)T * N * 3 * sizeof(Real);
  const Real* d_raw = unwrapped;
  const Real* d_raw_w = nullptr;
  if (!device_src) {
    Real* st = (Real*)ctx->staging.reserve(raw_bytes * (wrapped ? 2 : 1));
    AMDAT_CUDA(cudaMemcpyAsync(st, unwrapped, raw_bytes, cudaMemcpyHostToDevice, ctx->stream));
    d_raw = st;
    if (wrapped) {
      AMDAT_CUDA(cudaMemcpyAsync(st + (size_t)T * N * 3, wrapped, raw_bytes,
                                 cudaMemcpyHostToDevice, ctx->stream));
      d_raw_w = st + (size_t)T * N * 3;
    }
  }
  const float3 b = make_float3(box[0], box[1], box[2]);
  const float3 l = box_lo ? make_float3(box_lo[0], box_lo[1], box_lo[2]) : make_float3(0, 0, 0);
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>(ceil_div((int64_t)T * N, threads), (int64_t)ctx->n_sm * 16);
  stage_kernel<Real><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
      d_raw, d_raw_w, T, N, n_pad, b, l, ctx->u.ptr, ctx->w.ptr);
  check_launch("stage_kernel");
  count_launch(ctx);
  ctx->n_frames = T;
  ctx->n_atoms = N;
  ctx->n_pad = n_pad;
  std::memcpy(ctx->box, box, sizeof(ctx->box));
  if (box_lo) std::memcpy(ctx->box_lo, box_lo, sizeof(ctx->box_lo));
  else std::memset(ctx->box_lo, 0, sizeof(ctx->box_lo));
  for (auto& kv : ctx->pair_cache) delete kv.second;
  ctx->pair_cache.clear();
  ctx->disp_cache.clear();
  ++ctx->traj_serial;
  AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->have_traj = true;
  // list 0 = all atoms (contiguous); lists of a trajectory with another atom
  // count no longer apply and are dropped
  if (ctx->lists.empty()) ctx->lists.push_back(new ListEntry());
  if (ctx->lists[0]->n != N) {
    for (size_t i = 1; i < ctx->lists.size(); ++i) delete ctx->lists[i];
    ctx->lists.resize(1);
  }
  ctx->lists[0]->n = N;
  ctx->lists[0]->first = 0;
  ctx->lists[0]->contiguous = true;
}

}  // namespace amdat

using namespace amdat;

amdat_ctx::~amdat_ctx() {
  disp_cache.clear();
  for (auto* l : lists) delete l;
  for (auto& kv : pair_cache) delete kv.second;
  for (auto& kv : densities) {
    delete kv.second->rho;
    delete kv.second;
  }
  for (auto* b : rho_pool) delete b;
  for (auto& kv : bin_maps) delete kv.second;
  amdat::lattice_plans_free(this);
  amdat::sk_adjoint_plans_free(this);
  for (auto& r : prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : event_pool) cudaEventDestroy(e);
  if (own_stream) cudaStreamDestroy(own_stream);
}

namespace amdat {

DevBuf<float2>* rho_acquire(amdat_ctx* ctx, size_t count) {
  // smallest pooled buffer that fits, else a new one
  int best = -1;
  for (int i = 0; i < (int)ctx->rho_pool.size(); ++i)
    if (ctx->rho_pool[i]->n >= count && (best < 0 || ctx->rho_pool[i]->n < ctx->rho_pool[best]->n))
      best = i;
  if (best >= 0) {
    DevBuf<float2>* b = ctx->rho_pool[best];
    ctx->rho_pool.erase(ctx->rho_pool.begin() + best);
    return b;
  }
  auto* b = new DevBuf<float2>();
  try {
    b->reserve(count);
  } catch (...) {
    // free the pool and retry once before giving up
    for (auto* q : ctx->rho_pool) delete q;
    ctx->rho_pool.clear();
    try {
      b->reserve(count);
    } catch (...) {
      delete b;
      throw;
    }
  }
  return b;
}

void rho_release(amdat_ctx* ctx, DevBuf<float2>* b) {
  if (b) ctx->rho_pool.push_back(b);
}

static cudaEvent_t take_event(amdat_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  AMDAT_CUDA(cudaEventCreate(&e));
  return e;
}

KernelTimer::KernelTimer(amdat_ctx* c, const char* n) : ctx(c), name(n) {
  if (!ctx->profiling) return;
  a = take_event(ctx);
  b = take_event(ctx);
  cudaEventRecord(a, ctx->stream);
}

KernelTimer::~KernelTimer() {
  if (!a) return;
  cudaEventRecord(b, ctx->stream);
  ctx->prof_pending.push_back(ProfRec{name, a, b});
}

static void prof_collect(amdat_ctx* ctx) {
  for (auto& r : ctx->prof_pending) {
    float ms = 0.f;
    AMDAT_CUDA(cudaEventSynchronize(r.b));
    AMDAT_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    auto& st = ctx->prof_stats[r.name];
    st.first += 1;
    st.second += ms;
    ctx->event_pool.push_back(r.a);
    ctx->event_pool.push_back(r.b);
  }
  ctx->prof_pending.clear();
}

}  // namespace amdat

// FP64 planes for the plain path: the stored FP32 planes promoted to FP64 at
// first use (displacements u(t1) - u(t0) and wrapped positions are then
// formed in FP64 from the same values the mixed path reads).
namespace amdat {
__global__ void promote_kernel(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}
void ensure_fp64(amdat_ctx* ctx) {
  if (ctx->u64.ptr) return;
  const int64_t n = (int64_t)ctx->n_frames * 3 * ctx->n_pad;
  ctx->u64.reserve(n);
  ctx->w64.reserve(n);
  const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->n_sm * 16);
  promote_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(ctx->u.ptr, ctx->u64.ptr, n);
  promote_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(ctx->w.ptr, ctx->w64.ptr, n);
  check_launch("promote_kernel");
  count_launch(ctx, 2);
}
}  // namespace amdat

extern "C" {

const char* amdat_version(void) { return "amdat_gb300 0.1.0"; }
const char* amdat_last_error(void) { return g_last_error.c_str(); }

amdat_status amdat_create(int32_t device, amdat_ctx** out) {
  return guarded([&] {
    AMDAT_REQUIRE(out != nullptr, "null output pointer");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) throw Error(AMDAT_ERR_NO_DEVICE, "no CUDA device available");
    AMDAT_REQUIRE(device >= 0 && device < n, "device index out of range");
    auto* c = new amdat_ctx();
    c->device = device;
    try {
      AMDAT_CUDA(cudaSetDevice(device));
      AMDAT_CUDA(cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device));
      AMDAT_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
      c->stream = c->own_stream;
      c->lists.push_back(new ListEntry());
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

amdat_status amdat_destroy(amdat_ctx* ctx) {
  return guarded([&] {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete ctx;
  });
}

amdat_status amdat_set_stream(amdat_ctx* ctx, void* s) {
  return guarded([&] {
    check_ctx(ctx);
    ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
  });
}

amdat_status amdat_synchronize(amdat_ctx* ctx) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

amdat_status amdat_launch_count(amdat_ctx* ctx, int64_t* count) {
  return guarded([&] {
    AMDAT_REQUIRE(ctx && count, "null argument");
    *count = ctx->launches;
  });
}

amdat_status amdat_traj_upload(amdat_ctx* ctx, int32_t T, int32_t N, const float* unwrapped,
                               const float* wrapped, const float* box, const float* box_lo) {
  return guarded([&] {
    check_ctx(ctx);
    upload_impl<float>(ctx, T, N, unwrapped, wrapped, false, box, box_lo);
  });
}

amdat_status amdat_traj_upload_f64(amdat_ctx* ctx, int32_t T, int32_t N, const double* unwrapped,
                                   const double* wrapped, const float* box, const float* box_lo) {
  return guarded([&] {
    check_ctx(ctx);
    upload_impl<double>(ctx, T, N, unwrapped, wrapped, false, box, box_lo);
  });
}

amdat_status amdat_traj_upload_device(amdat_ctx* ctx, int32_t T, int32_t N,
                                      const float* d_unwrapped, const float* box,
                                      const float* box_lo) {
  return guarded([&] {
    check_ctx(ctx);
    upload_impl<float>(ctx, T, N, d_unwrapped, nullptr, true, box, box_lo);
  });
}

amdat_status amdat_list_create(amdat_ctx* ctx, const int32_t* atoms, int32_t n, int32_t* handle) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(handle != nullptr, "null handle pointer");
    if (!ctx->have_traj) throw Error(AMDAT_ERR_STATE, "upload a trajectory before creating lists");
    AMDAT_REQUIRE(n >= 0 && (n == 0 || atoms != nullptr), "bad list");
    for (int32_t i = 0; i < n; ++i) {
      AMDAT_REQUIRE(atoms[i] >= 0 && atoms[i] < ctx->n_atoms, "list atom index out of range");
      AMDAT_REQUIRE(i == 0 || atoms[i] > atoms[i - 1], "list atoms must be strictly ascending");
    }
    auto* e = new ListEntry();
    e->n = n;
    e->contiguous = (n == 0) || (atoms[n - 1] - atoms[0] == n - 1);
    e->first = n ? atoms[0] : 0;
    if (!e->contiguous) {
      e->idx.reserve(n);
      AMDAT_CUDA(cudaMemcpy(e->idx.ptr, atoms, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    }
    ctx->lists.push_back(e);
    *handle = (int32_t)ctx->lists.size() - 1;
  });
}

amdat_status amdat_list_size(amdat_ctx* ctx, int32_t handle, int32_t* n) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(n != nullptr, "null output");
    *n = list_entry(ctx, handle).n;
  });
}

amdat_status amdat_profile_reset(amdat_ctx* ctx, int32_t enable) {
  return guarded([&] {
    check_ctx(ctx);
    prof_collect(ctx);
    ctx->prof_stats.clear();
    ctx->profiling = enable != 0;
  });
}

amdat_status amdat_profile_kernel(amdat_ctx* ctx, const char* kernel, int64_t* launches,
                                  double* total_ms) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(kernel != nullptr, "null kernel name");
    prof_collect(ctx);
    auto it = ctx->prof_stats.find(kernel);
    if (launches) *launches = it == ctx->prof_stats.end() ? 0 : it->second.first;
    if (total_ms) *total_ms = it == ctx->prof_stats.end() ? 0.0 : it->second.second;
  });
}

amdat_status amdat_set_scheme(amdat_ctx* ctx, const amdat_scheme* s) {
  return guarded([&] {
    check_ctx(ctx);
    AMDAT_REQUIRE(s != nullptr, "null scheme");
    scheme_check(*s);
    ctx->scheme = *s;
    ctx->have_scheme = true;
    ++ctx->scheme_serial;
    ctx->disp_cache.clear();
    for (auto& kv : ctx->pair_cache) delete kv.second;
    ctx->pair_cache.clear();
  });
}

}  // extern "C"
