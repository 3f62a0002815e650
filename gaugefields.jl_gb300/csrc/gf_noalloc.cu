// gf_plaquette_noalloc: the plaquette sum for callers that must not allocate
// device memory.
//
// Some callers cannot call cudaMalloc: an application whose device memory is
// owned by another allocator (Julia's CUDA.jl pool, PyTorch's caching
// allocator) that must account for every byte, or a time-critical loop where a
// cudaMalloc would synchronise the device. gf_plaquette needs a context, and
// creating one allocates its reduction buffer; this entry point instead keeps
// its per-block partial sums in a fixed file-scope device array.
//
// The array is GF_NOALLOC_MAX_BLOCKS doubles (1 MiB). Every GPU that loads the
// library holds it until the process exits. One block reduces 128 sites, so
// the largest lattice is 128 * GF_NOALLOC_MAX_BLOCKS = 16,777,216 sites (64^4);
// larger volumes are rejected with GF_EINVAL.
//
// Every call shares the array and overwrites the partials it uses, so calls
// whose kernels overlap on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the caller.
//
// In host code the array's name is only a host-side stand-in; the device
// address is looked up with cudaGetSymbolAddress once per device, with that
// device current, by the first call on the device. That first call should be
// made before any stream capture begins. The address is kept for the life of
// the process: after cudaDeviceReset (or any teardown of the device's primary
// context) the kept address is stale, so this entry point must not be called
// again in a process that has reset the device.
#include "gf_internal.h"
#include "stencil.cuh"
#include <mutex>

#define GF_NOALLOC_MAX_BLOCKS 131072
#define GF_NOALLOC_BLOCK 128
#define GF_NOALLOC_MAX_DEVICES 64

namespace gf {

static __device__ __align__(256) double g_noalloc_partials[GF_NOALLOC_MAX_BLOCKS];

__global__ void __launch_bounds__(GF_NOALLOC_BLOCK)
    k_plaquette_noalloc(LinkSrc<double, false> U, Geom g, double* __restrict__ part) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < g.vol) {
    Site st = site_of(g, s);
    v = plaq_site<double>(U, g, st, s);
  }
  block_partial_sum(v, part);
}

__global__ void k_noalloc_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) *out = v;
  }
}

static std::mutex g_noalloc_mu;
static double* g_noalloc_addr[GF_NOALLOC_MAX_DEVICES];

// Device address of the partials array on the current device (set-up on the
// first call per device).
static cudaError_t noalloc_scratch(int dev, double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = (double*)p;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

}  // namespace gf

// the message is returned by gf_last_error(NULL)
static int noalloc_fail(int code, const std::string& m) {
  gf::set_global_error(m);
  return code;
}

extern "C" int gf_plaquette_noalloc(const void* links, const int L[4], double* out, void* stream) {
  using namespace gf;
  if (!links || !L || !out) return noalloc_fail(GF_EINVAL, "gf_plaquette_noalloc: null argument");
  // The volume is checked against the limit after every factor, so the
  // product never overflows (each extent is below 2^31 and the running
  // product at most 2^24 before the next multiply).
  const long long vmax = (long long)GF_NOALLOC_MAX_BLOCKS * GF_NOALLOC_BLOCK;
  long long V = 1;
  for (int i = 0; i < 4; ++i) {
    if (L[i] < 2 || (L[i] % 2) != 0)
      return noalloc_fail(GF_EINVAL, "gf_plaquette_noalloc: every lattice extent must be even and >= 2");
    V *= L[i];
    if (V > vmax)
      return noalloc_fail(GF_EINVAL, "gf_plaquette_noalloc: lattice has more than " + std::to_string(vmax) +
                                         " sites; the fixed scratch holds at most " + std::to_string(vmax));
  }
  long long nb = (V + GF_NOALLOC_BLOCK - 1) / GF_NOALLOC_BLOCK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(GF_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= GF_NOALLOC_MAX_DEVICES) return noalloc_fail(GF_EINVAL, "gf_plaquette_noalloc: device ordinal too large");
  double* part = nullptr;
  e = noalloc_scratch(dev, &part);
  if (e != cudaSuccess) return noalloc_fail(GF_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  Geom g;
  for (int i = 0; i < 4; ++i) g.L[i] = L[i];
  g.vol = (int)V;
  g.vh = (int)(V / 2);
  g.stride[0] = 1;
  g.stride[1] = L[0];
  g.stride[2] = L[0] * L[1];
  g.stride[3] = L[0] * L[1] * L[2];
  cudaStream_t s = (cudaStream_t)stream;
  LinkSrc<double, false> src{(const double2*)links};
  k_plaquette_noalloc<<<(unsigned)nb, GF_NOALLOC_BLOCK, 0, s>>>(src, g, part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(GF_ECUDA, std::string("plaquette launch: ") + cudaGetErrorString(e));
  k_noalloc_final<<<1, 1024, 0, s>>>(part, (int)nb, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(GF_ECUDA, std::string("reduction launch: ") + cudaGetErrorString(e));
  return GF_OK;
}
