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

}  // namespace gf
