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
#include <cstdlib>
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

// ---------------------------------------------------------------------------
// cell lists for short-range ordered pair loops (the distinct van Hove pass and
// RDFs of two different lists): when every box axis holds at least three cells
// no narrower than the last bin edge, a pair that can fall in a bin has its
// atoms in the same or neighbouring cells (periodic).  Per frame the list's
// atoms are counted into cells, the counts scanned and the atoms scattered in
// cell order as (x, y, z, atom index bits); a thread takes one list-1 member in
// cell order at t0 and visits the 27 cells around it in the list-2 cells at t1.
// Distances and bins are the exact chain of pair_term, counts are integer
// atomics, so the counts equal the all-pairs kernel's bit for bit.
// ---------------------------------------------------------------------------
struct PHCells {
  int3 nc;
  float3 lo, inv_cell;
  int32_t n_cells;
  const int32_t* start;  // [slot][n_cells + 1]
  const float4* pos;     // [slot][n]: members in cell order
  int32_t n;             // members per slot
};

__device__ __forceinline__ int ph_cell_axis(float x, float lo, float inv_cell, int n) {
  const int c = (int)((x - lo) * inv_cell);
  return min(max(c, 0), n - 1);
}

// members of list l at frame frames[s] counted into the cells of slot s
__global__ void ph_cell_count_kernel(const float* __restrict__ w, int64_t n_pad, PHList l,
                                     const int32_t* __restrict__ frames, int3 nc, float3 lo, float3 inv_cell,
                                     int32_t* __restrict__ cell_of, int32_t* __restrict__ count) {
  const int s = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= l.n) return;
  const float* P = w + (int64_t)frames[s] * 3 * n_pad;
  const int a = member(l, i);
  const int c = (ph_cell_axis(P[2 * n_pad + a], lo.z, inv_cell.z, nc.z) * nc.y +
                 ph_cell_axis(P[n_pad + a], lo.y, inv_cell.y, nc.y)) * nc.x +
                ph_cell_axis(P[a], lo.x, inv_cell.x, nc.x);
  cell_of[(int64_t)s * l.n + i] = c;
  atomicAdd(count + (int64_t)s * nc.x * nc.y * nc.z + c, 1);
}

// exclusive scan of one slot's cell counts (one block per slot) into start and
// the scatter cursors
__global__ void __launch_bounds__(1024) ph_cell_scan_kernel(const int32_t* __restrict__ count, int32_t n_cells,
                                                            int32_t* __restrict__ start, int32_t* __restrict__ cursor) {
  __shared__ int32_t s_part[1024];
  __shared__ int32_t s_carry;
  const int s = blockIdx.x;
  const int32_t* C = count + (int64_t)s * n_cells;
  int32_t* S = start + (int64_t)s * (n_cells + 1);
  int32_t* U = cursor + (int64_t)s * n_cells;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < n_cells; base += 1024) {
    const int i = base + threadIdx.x;
    s_part[threadIdx.x] = i < n_cells ? C[i] : 0;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int v = threadIdx.x >= off ? s_part[threadIdx.x - off] : 0;
      __syncthreads();
      s_part[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < n_cells) {
      const int excl = s_carry + s_part[threadIdx.x] - C[i];
      S[i] = excl;
      U[i] = excl;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_carry += s_part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) S[n_cells] = s_carry;
}

__global__ void ph_cell_scatter_kernel(const float* __restrict__ w, int64_t n_pad, PHList l,
                                       const int32_t* __restrict__ frames, int32_t n_cells,
                                       const int32_t* __restrict__ cell_of, int32_t* __restrict__ cursor,
                                       float4* __restrict__ pos) {
  const int s = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= l.n) return;
  const float* P = w + (int64_t)frames[s] * 3 * n_pad;
  const int a = member(l, i);
  const int k = atomicAdd(cursor + (int64_t)s * n_cells + cell_of[(int64_t)s * l.n + i], 1);
  pos[(int64_t)s * l.n + k] = make_float4(P[a], P[n_pad + a], P[2 * n_pad + a], __int_as_float(a));
}

// ordered pairs (i at t0 from list 1, j != i at t1 from list 2) within the 27
// cells around i; slot_a / slot_b give each row's cell slots
__global__ void __launch_bounds__(PH_THREADS)
    pair_hist_cells_kernel(PHParams p, PHCells C1, PHCells C2, const int32_t* __restrict__ slot_a,
                           const int32_t* __restrict__ slot_b) {
  extern __shared__ unsigned int sh_hist[];  // [8 warps][n_bins]
  const int q = blockIdx.y;
  const int warp = threadIdx.x >> 5;
  unsigned int* hist = sh_hist + warp * p.n_bins;
  for (int b = threadIdx.x; b < 8 * p.n_bins; b += blockDim.x) sh_hist[b] = 0u;
  __syncthreads();
  const int i = blockIdx.x * PH_THREADS + threadIdx.x;
  if (i < C1.n) {
    const float4 pi = C1.pos[(int64_t)slot_a[q] * C1.n + i];
    const int ai = __float_as_int(pi.w);
    const int32_t* S2 = C2.start + (int64_t)slot_b[q] * (C2.n_cells + 1);
    const float4* P2 = C2.pos + (int64_t)slot_b[q] * C2.n;
    const int cx = ph_cell_axis(pi.x, C2.lo.x, C2.inv_cell.x, C2.nc.x);
    const int cy = ph_cell_axis(pi.y, C2.lo.y, C2.inv_cell.y, C2.nc.y);
    const int cz = ph_cell_axis(pi.z, C2.lo.z, C2.inv_cell.z, C2.nc.z);
    for (int dz = -1; dz <= 1; ++dz) {
      int z = cz + dz;
      z += z < 0 ? C2.nc.z : (z >= C2.nc.z ? -C2.nc.z : 0);
      for (int dy = -1; dy <= 1; ++dy) {
        int y = cy + dy;
        y += y < 0 ? C2.nc.y : (y >= C2.nc.y ? -C2.nc.y : 0);
        for (int dx = -1; dx <= 1; ++dx) {
          int x = cx + dx;
          x += x < 0 ? C2.nc.x : (x >= C2.nc.x ? -C2.nc.x : 0);
          const int c = (z * C2.nc.y + y) * C2.nc.x + x;
          const int k1 = __ldg(S2 + c + 1);
          for (int k = __ldg(S2 + c); k < k1; ++k) {
            const float4 cj = __ldg(P2 + k);
            if (__float_as_int(cj.w) != ai) pair_term<false>(p, cj, pi.x, pi.y, pi.z, hist, 1u);
          }
        }
      }
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
  // cell lists for the ordered pass when the box holds at least three cells per
  // axis no narrower than the last bin edge (with a 1e-4 margin over the
  // in-range cut, so a rounding of a cell index never splits an in-range pair)
  const float cell_edge = (float)((double)max_distance * (1.0 + 1e-4));
  const int3 nc = make_int3((int)std::floor(ctx->box[0] / cell_edge), (int)std::floor(ctx->box[1] / cell_edge),
                            (int)std::floor(ctx->box[2] / cell_edge));
  const int64_t n_cells = (int64_t)nc.x * nc.y * nc.z;
  const char* pc = std::getenv("AMDAT_PAIR_CELLS");  // "off": the all-pairs pass
  const bool cells = !symmetric && n_q && l1.n > 0 && l2.n >= 1024 && nc.x >= 3 && nc.y >= 3 && nc.z >= 3 &&
                     n_cells <= (1 << 20) && !(pc && std::strcmp(pc, "off") == 0);
  if (cells) {
    // frame slots: the distinct frames of each side; one structure when both
    // sides are the same list
    const bool same = &l1 == &l2;
    std::vector<int32_t> fr1, fr2;
    auto slots = [](const std::vector<int32_t>& f, std::vector<int32_t>& uniq, std::vector<int32_t>& slot_of) {
      uniq = f;
      std::sort(uniq.begin(), uniq.end());
      uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
      slot_of.resize(f.size());
      for (size_t i = 0; i < f.size(); ++i)
        slot_of[i] = (int32_t)(std::lower_bound(uniq.begin(), uniq.end(), f[i]) - uniq.begin());
    };
    std::vector<int32_t> sa, sb;
    if (same) {
      std::vector<int32_t> both(fa);
      both.insert(both.end(), fb.begin(), fb.end());
      std::vector<int32_t> tmp;
      slots(both, fr1, tmp);
      sa.assign(tmp.begin(), tmp.begin() + (std::ptrdiff_t)n_q);
      sb.assign(tmp.begin() + (std::ptrdiff_t)n_q, tmp.end());
      fr2 = fr1;
    } else {
      slots(fa, fr1, sa);
      slots(fb, fr2, sb);
    }
    const int n_sides = same ? 1 : 2;
    const ListEntry* lists[2] = {&l1, &l2};
    const std::vector<int32_t>* frs[2] = {&fr1, &fr2};
    size_t need = 0;
    size_t off[2][6];
    for (int s = 0; s < n_sides; ++s) {
      const size_t nf = frs[s]->size(), n = (size_t)lists[s]->n;
      off[s][0] = need; need = align(need + nf * 4);                           // frames
      off[s][1] = need; need = align(need + nf * n * 4);                       // cell_of
      off[s][2] = need; need = align(need + nf * (size_t)n_cells * 4);         // count
      off[s][3] = need; need = align(need + nf * (size_t)(n_cells + 1) * 4);   // start
      off[s][4] = need; need = align(need + nf * (size_t)n_cells * 4);         // cursor
      off[s][5] = need; need = align(need + nf * n * sizeof(float4));          // pos
    }
    const size_t o_sa = need; need = align(need + n_q * 4);
    const size_t o_sb = need; need = align(need + n_q * 4);
    unsigned char* cb = ctx->scratch2.reserve(need);
    cudaStream_t st = ctx->stream;
    AMDAT_CUDA(cudaMemcpyAsync(cb + o_sa, sa.data(), n_q * 4, cudaMemcpyHostToDevice, st));
    AMDAT_CUDA(cudaMemcpyAsync(cb + o_sb, sb.data(), n_q * 4, cudaMemcpyHostToDevice, st));
    PHCells C[2];
    for (int s = 0; s < n_sides; ++s) {
      const int nf = (int)frs[s]->size();
      const PHList l = phview(*lists[s]);
      PHCells& c = C[s];
      c.nc = nc;
      c.lo = make_float3(ctx->box_lo[0], ctx->box_lo[1], ctx->box_lo[2]);
      c.inv_cell = make_float3((float)nc.x / ctx->box[0], (float)nc.y / ctx->box[1], (float)nc.z / ctx->box[2]);
      c.n_cells = (int32_t)n_cells;
      c.start = (const int32_t*)(cb + off[s][3]);
      c.pos = (const float4*)(cb + off[s][5]);
      c.n = l.n;
      AMDAT_CUDA(cudaMemcpyAsync(cb + off[s][0], frs[s]->data(), (size_t)nf * 4, cudaMemcpyHostToDevice, st));
      AMDAT_CUDA(cudaMemsetAsync(cb + off[s][2], 0, (size_t)nf * n_cells * 4, st));
      AMDAT_REQUIRE(nf <= 65535, "at most 65535 frames per call");
      const dim3 g((unsigned)ceil_div(l.n, 256), (unsigned)nf);
      ph_cell_count_kernel<<<g, 256, 0, st>>>(p.w, p.n_pad, l, (const int32_t*)(cb + off[s][0]), nc, c.lo,
                                              c.inv_cell, (int32_t*)(cb + off[s][1]), (int32_t*)(cb + off[s][2]));
      ph_cell_scan_kernel<<<(unsigned)nf, 1024, 0, st>>>((const int32_t*)(cb + off[s][2]), (int32_t)n_cells,
                                                          (int32_t*)(cb + off[s][3]), (int32_t*)(cb + off[s][4]));
      ph_cell_scatter_kernel<<<g, 256, 0, st>>>(p.w, p.n_pad, l, (const int32_t*)(cb + off[s][0]), (int32_t)n_cells,
                                                (const int32_t*)(cb + off[s][1]), (int32_t*)(cb + off[s][4]),
                                                (float4*)(cb + off[s][5]));
      check_launch("pair cell lists");
      count_launch(ctx, 3);
    }
    if (same) C[1] = C[0];
    const size_t shm = (size_t)8 * n_bins * 4;
    if (shm > 48 * 1024)
      AMDAT_CUDA(cudaFuncSetAttribute(pair_hist_cells_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    AMDAT_REQUIRE(n_q <= 65535, "at most 65535 frames or time pairs per call");
    dim3 grid((unsigned)ceil_div(l1.n, PH_THREADS), (unsigned)n_q);
    KernelTimer kt(ctx, "pair_hist_cells_kernel");
    pair_hist_cells_kernel<<<grid, PH_THREADS, shm, st>>>(p, C[0], C[1], (const int32_t*)(cb + o_sa),
                                                          (const int32_t*)(cb + o_sb));
    check_launch("pair_hist_cells_kernel");
    count_launch(ctx);
  } else if (n_q && l1.n > 0 && l2.n > 0) {
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
