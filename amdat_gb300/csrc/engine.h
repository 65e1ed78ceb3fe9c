// Internal state of an amdat_gb300 context (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/amdat_gb300.h"

namespace amdat {

// Errors inside the engine are C++ exceptions carrying an amdat_status; the
// ABI wrappers turn them into return codes plus a thread-local message.
struct Error : std::runtime_error {
  amdat_status status;
  Error(amdat_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string& msg);

#define AMDAT_REQUIRE(cond, msg)                                       \
  do {                                                                 \
    if (!(cond)) throw ::amdat::Error(AMDAT_ERR_ARGUMENT, (msg));      \
  } while (0)

#define AMDAT_CUDA(call)                                                              \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      throw ::amdat::Error(e_ == cudaErrorMemoryAllocation ? AMDAT_ERR_MEMORY         \
                                                           : AMDAT_ERR_CUDA,          \
                           std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

template <class F>
amdat_status guarded(F&& f) {
  try {
    f();
    return AMDAT_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return AMDAT_ERR_MEMORY;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return AMDAT_ERR_ARGUMENT;
  }
}

// ---------------------------------------------------------------------------
// time scheme (host)
// ---------------------------------------------------------------------------
struct Pairs {
  std::vector<int32_t> gap, t0, t1;
  std::vector<int32_t> gap_first;  // [n_gaps + 1]: pairs of gap g are gap_first[g]..gap_first[g+1]
};
int32_t scheme_n_timesteps(const amdat_scheme& s);
int32_t scheme_n_timegaps(const amdat_scheme& s);
Pairs scheme_pairs(const amdat_scheme& s, bool fullblock, bool loop_order);
void scheme_check(const amdat_scheme& s);

// ---------------------------------------------------------------------------
// device memory owned by a context
// ---------------------------------------------------------------------------
template <class T>
struct DevBuf {
  T* ptr = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    n = 0;
  }
  // grow-only: keeps the allocation when it is already large enough
  T* reserve(size_t count) {
    if (count <= n && ptr) return ptr;
    release();
    if (count == 0) count = 1;
    AMDAT_CUDA(cudaMalloc(&ptr, count * sizeof(T)));
    n = count;
    return ptr;
  }
};

struct ListEntry {
  int32_t n = 0;
  int32_t first = 0;          // contiguous lists: atoms first..first+n-1
  bool contiguous = true;
  DevBuf<int32_t> idx;        // gathered lists: ascending atom indices
};

struct PairTable {
  int64_t n_pairs = 0;
  int32_t n_gaps = 0;
  std::vector<int32_t> gap_first;
  DevBuf<int32_t> t0, t1, gap;
  std::vector<int32_t> h_t0, h_t1, h_gap;  // host copies (plan tables resolve pairs on the host)
  // lagged tables (linear schemes): every gap's pairs, in order, are
  // (t, t + lag[g]) for t = 0 .. count - 1
  bool lagged = false;
  std::vector<int32_t> lag;
};

struct LatticePlanDev;
struct SkAdjointPlan;

// Spatial bins of the wrapped coordinates: flat bin (ix * ny + iy) * nz + iz of
// every atom in every frame, -1 outside the binned region
struct BinMap {
  int32_t nx = 0, ny = 0, nz = 0;
  int32_t n_frames = 0, n_pad = 0;  // trajectory shape the map was made for
  DevBuf<int32_t> bin;              // [frames][n_pad]
};

struct Density {
  int32_t list = 0;
  int32_t n_k = 0;
  int32_t n_frames = 0;
  int32_t n_shells = 0;
  float period = 0.f;              // k = 2 pi n / period
  int32_t n_list = 0;              // list size when the density was computed
  std::string lattice_key;         // lattice densities: the plan key (kmax, dk, period)
  std::vector<int32_t> frames;     // system frame of each row
  std::vector<int32_t> kvec;       // [3*n_k] (lattice mode: shell-sorted)
  std::vector<int32_t> shell_off;  // lattice mode
  DevBuf<float2>* rho = nullptr;   // [n_frames][n_k], from the context's pool
};

// per-kernel CUDA-event timing (amdat_profile_*)
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};

}  // namespace amdat

struct amdat_ctx {
  int device = 0;
  int n_sm = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;

  // trajectory (FP32 structure-of-arrays planes [frame][xyz][n_pad])
  int32_t n_frames = 0, n_atoms = 0, n_pad = 0;
  float box[3] = {0, 0, 0}, box_lo[3] = {0, 0, 0};
  amdat::DevBuf<float> u;      // unwrapped, re-referenced to frame 0
  amdat::DevBuf<float> w;      // wrapped
  amdat::DevBuf<double> u64;   // unwrapped FP64 (plain path), raw coordinates
  amdat::DevBuf<double> w64;   // wrapped FP64 (plain path)
  bool have_traj = false;

  std::vector<amdat::ListEntry*> lists;
  amdat_scheme scheme{};
  bool have_scheme = false;
  uint64_t scheme_serial = 0;  // bumped by every amdat_set_scheme (plans bake pair frames)
  uint64_t traj_serial = 0;    // bumped by every trajectory upload
  // one-shot displacement runs keep their prepared plans, keyed by the whole
  // request (scheme and trajectory serials included), most recent last
  std::vector<std::pair<std::string, std::shared_ptr<amdat_disp_plan>>> disp_cache;
  std::map<int, amdat::PairTable*> pair_cache;  // key: fullblock*2 + loop_order
  std::map<int32_t, amdat::Density*> densities;
  int32_t next_density = 1;
  std::map<int32_t, amdat::BinMap*> bin_maps;
  int32_t next_bins = 1;

  // scratch reused across calls
  amdat::DevBuf<unsigned char> scratch;
  amdat::DevBuf<unsigned char> scratch2;
  amdat::DevBuf<unsigned char> staging;
  std::vector<amdat::DevBuf<float2>*> rho_pool;        // released density tables
  std::map<std::string, amdat::LatticePlanDev*> lattice_plans;
  std::map<std::string, amdat::SkAdjointPlan*> sk_adjoint_plans;  // by lattice key

  bool profiling = false;
  std::vector<amdat::ProfRec> prof_pending;
  std::vector<cudaEvent_t> event_pool;
  std::map<std::string, std::pair<int64_t, double>> prof_stats;  // launches, total ms

  ~amdat_ctx();
};

namespace amdat {
amdat_ctx* check_ctx(amdat_ctx* ctx);
const PairTable& pair_table(amdat_ctx* ctx, bool fullblock, bool loop_order);
const ListEntry& list_entry(amdat_ctx* ctx, int32_t handle);
Density& density(amdat_ctx* ctx, int32_t handle);
void ensure_fp64(amdat_ctx* ctx);
void count_launch(amdat_ctx* ctx, int n = 1);
void check_launch(const char* what);
DevBuf<float2>* rho_acquire(amdat_ctx* ctx, size_t count);
void rho_release(amdat_ctx* ctx, DevBuf<float2>* b);
void lattice_plans_free(amdat_ctx* ctx);
void sk_adjoint_plans_free(amdat_ctx* ctx);
void fixed_turns_launch(amdat_ctx* ctx, const int32_t* d_frames, int32_t n_frames, const ListEntry& e,
                        float period, int4* out);

// RAII event pair around one kernel launch when profiling is enabled
struct KernelTimer {
  amdat_ctx* ctx;
  const char* name;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelTimer(amdat_ctx* c, const char* n);
  ~KernelTimer();
};
inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
}  // namespace amdat
