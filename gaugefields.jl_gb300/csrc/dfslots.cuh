// Per-thread shared-memory slots of the double-float table kernels: slot k
// of a thread holds one double-float 3x3 matrix as 9 float4 (re.hi, re.lo,
// im.hi, im.lo), element-major over the 128 threads of a block, so a warp's
// 128-bit accesses cover consecutive banks (36 floats per thread and slot).
#pragma once
#include "su3.cuh"

namespace gf {

__device__ __forceinline__ mat3<dfl> slot_load(const float* sm, int slot, int tid) {
  mat3<dfl> m;
  const float4* q = reinterpret_cast<const float4*>(sm) + slot * 9 * 128 + tid;
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    const float4 v = q[e * 128];
    m.e[e / 3][e % 3] = mk(dfl(v.x, v.y), dfl(v.z, v.w));
  }
  return m;
}
__device__ __forceinline__ void slot_store(float* sm, int slot, int tid, const mat3<dfl>& m) {
  float4* q = reinterpret_cast<float4*>(sm) + slot * 9 * 128 + tid;
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    const cplx<dfl> v = m.e[e / 3][e % 3];
    q[e * 128] = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo);
  }
}

// Table products leave their slot entries normalised (1) or as raw grid pairs
// (0): the value (A - K) + L with a low word of up to ~2^-19 of the product's
// bound. Products read raw pairs as accurately as normalised ones (the grid
// only sees high words); the operator arithmetic of the kernels' other code
// (Cayley-Hamilton coefficients, projections, scalings) loses accuracy on
// them, so that code and every store to a field read normalised values
// (slot_load_n). At 32^4 raw pairs measured 1.88 trajectories/s against 1.84
// (1.92 with GF_DF_DAG_LOAD = 1) at about 1.5 times the force error (the
// 16^4 stout force 1.4e-11 of the fp64 oracle's); the default keeps the
// accuracy.
#ifndef GF_DF_NORM
#define GF_DF_NORM 1
#endif
__device__ __forceinline__ mat3<dfl> df_normalise(const mat3<dfl>& m) {
  mat3<dfl> r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      r.e[i][j] = mk(df_fast_two_sum(m.e[i][j].re.hi, m.e[i][j].re.lo),
                     df_fast_two_sum(m.e[i][j].im.hi, m.e[i][j].im.lo));
  return r;
}
__device__ __forceinline__ mat3<dfl> slot_load_n(const float* sm, int slot, int tid) {
  return GF_DF_NORM ? slot_load(sm, slot, tid) : df_normalise(slot_load(sm, slot, tid));
}

}  // namespace gf
