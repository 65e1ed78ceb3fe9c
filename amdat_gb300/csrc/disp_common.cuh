// Device helpers shared by the displacement kernels: compensated FP32 sums and
// the fixed-point F_s phases (a displacement as an int32 fraction of a turn,
// 2^-31 turns per unit, so the phase of an integer lattice vector is an exact
// wrapping integer combination and only the final conversion rounds).
#pragma once

#include <cstdint>

#include "f32x2.cuh"

namespace amdat {

// --- compensated FP32 helpers ------------------------------------------------
struct KSum {
  float s, c;
};
__device__ __forceinline__ void kadd(KSum& k, float v) {
  float y = __fsub_rn(v, k.c);
  float t = __fadd_rn(k.s, y);
  k.c = __fsub_rn(__fsub_rn(t, k.s), y);
  k.s = t;
}
// error-free sum of two compensated values (TwoSum of the leading parts)
__device__ __forceinline__ KSum kmerge(KSum a, KSum b) {
  float s = __fadd_rn(a.s, b.s);
  float bb = __fsub_rn(s, a.s);
  float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(b.s, bb));
  // a KSum holds the value s - c: (a.s - a.c) + (b.s - b.c) = s + err - a.c - b.c
  KSum r;
  r.s = s;
  r.c = __fsub_rn(__fadd_rn(a.c, b.c), err);
  return r;
}
__device__ __forceinline__ KSum kshfl(KSum v, int off) {
  KSum o;
  o.s = __shfl_down_sync(0xffffffffu, v.s, off);
  o.c = __shfl_down_sync(0xffffffffu, v.c, off);
  return o;
}

// fraction of a turn dr/L, as int32 in units of 2^-31 turns (exact wrap)
__device__ __forceinline__ int32_t turns_fixed(float d, float period) {
  float t = __fdiv_rn(d, period);
  t = __fsub_rn(t, rintf(t));  // [-0.5, 0.5]
  return __float2int_rn(__fmul_rn(t, 2147483648.0f));
}
// |d|^2 in the displacement kernels' fixed order: fma(z, z, fma(y, y, x * x))
__device__ __forceinline__ float sq3(float x, float y, float z) { return fmaf(z, z, fmaf(y, y, x * x)); }

// cos(2 pi * phase * 2^-31)
__device__ __forceinline__ float cos_fixed(int32_t phase) {
  return cospif(__fmul_rn((float)phase, 9.313225746154785e-10f));  // 2^-30
}

// cos of the same fixed-point phase through the SFU cosine: the phase is first
// reduced to [-1/2, 1/2) turn (a wrapping doubling of the int32: units of 2^-32
// turn), where __cosf's absolute error is below 2^-21.4
__device__ __forceinline__ float cos_fixed_sfu(int32_t phase) {
  const int32_t r = (int32_t)((uint32_t)phase << 1);
  return __cosf(__fmul_rn((float)r, 1.4629180792671596e-09f));  // 2 pi / 2^32
}
// the same cosine of a phase already doubled (units of 2^-32 turn, [-1/2, 1/2))
__device__ __forceinline__ float cos_turn32_sfu(int32_t r) {
  return __cosf(__fmul_rn((float)r, 1.4629180792671596e-09f));  // 2 pi / 2^32
}

// F_s of one displacement over a list of lattice vectors: the compensated sum
// of the cosines of the exact fixed-point phases, in blocks of 32 terms (each
// block summed plainly, then added to the compensated sum, and a closing empty
// block when the count is a multiple of 32), the vectors read from shared memory
// (SMEM) or through the read-only cache
template <bool SMEM>
__device__ __forceinline__ KSum list_shell_sum(const int4* R, int32_t fx, int32_t fy, int32_t fz, int v_begin,
                                               int v_end) {
  // n . (2 f) mod 2^32 is the doubled phase cos_fixed_sfu forms from n . f
  const uint32_t gx = (uint32_t)fx << 1, gy = (uint32_t)fy << 1, gz = (uint32_t)fz << 1;
  KSum acc = {0.f, 0.f};
  for (int v0 = v_begin; v0 < v_end; v0 += 32) {
    const int v1 = min(v0 + 32, v_end);
    float blk = 0.f;
#pragma unroll 4
    for (int v = v0; v < v1; ++v) {
      const int4 n = SMEM ? R[v] : __ldg(R + v);
      blk += cos_turn32_sfu((int32_t)((uint32_t)n.x * gx + (uint32_t)n.y * gy + (uint32_t)n.z * gz));
    }
    kadd(acc, blk);
  }
  if ((v_end - v_begin) % 32 == 0) kadd(acc, 0.f);  // the closing (empty) block
  return acc;
}

// list_shell_sum for two displacements at once (each vector read once for
// both; the scale multiply and the block sums as packed pairs).  Each result
// is the one list_shell_sum gives for that displacement, bit for bit.
template <bool SMEM>
__device__ __forceinline__ void list_shell_sum2(const int4* R, int32_t fxa, int32_t fya, int32_t fza, int32_t fxb,
                                                int32_t fyb, int32_t fzb, int v_begin, int v_end, KSum& acc_a,
                                                KSum& acc_b) {
  const uint32_t ax = (uint32_t)fxa << 1, ay = (uint32_t)fya << 1, az = (uint32_t)fza << 1;
  const uint32_t bx = (uint32_t)fxb << 1, by = (uint32_t)fyb << 1, bz = (uint32_t)fzb << 1;
  const uint64_t scale = pk2(1.4629180792671596e-09f, 1.4629180792671596e-09f);  // 2 pi / 2^32
  acc_a = KSum{0.f, 0.f};
  acc_b = KSum{0.f, 0.f};
  for (int v0 = v_begin; v0 < v_end; v0 += 32) {
    const int v1 = min(v0 + 32, v_end);
    uint64_t blk = 0ull;  // (0.f, 0.f)
#pragma unroll 4
    for (int v = v0; v < v1; ++v) {
      const int4 n = SMEM ? R[v] : __ldg(R + v);
      const int32_t pa = (int32_t)((uint32_t)n.x * ax + (uint32_t)n.y * ay + (uint32_t)n.z * az);
      const int32_t pb = (int32_t)((uint32_t)n.x * bx + (uint32_t)n.y * by + (uint32_t)n.z * bz);
      float xa, xb;
      upk2(mul2(pk2((float)pa, (float)pb), scale), xa, xb);
      blk = add2(blk, pk2(__cosf(xa), __cosf(xb)));
    }
    float ba, bb;
    upk2(blk, ba, bb);
    kadd(acc_a, ba);
    kadd(acc_b, bb);
  }
  if ((v_end - v_begin) % 32 == 0) {  // the closing (empty) block
    kadd(acc_a, 0.f);
    kadd(acc_b, 0.f);
  }
}

}  // namespace amdat
