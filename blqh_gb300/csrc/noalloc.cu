// SpMV that allocates no device memory.
//
// The regular SpMV path (blqh_spmv, and the one inside the Lanczos objects)
// allocates its working buffers with cudaMalloc. Some callers cannot do that:
// code that receives all of its device memory from a host framework's pool or
// arena, plugins loaded into a runtime that forbids allocation after start-up,
// and services that must not let an allocation synchronize the device in the
// middle of their own stream work. This file gives them one entry point,
// blqh_spmv_f32_noalloc, a variant of the double-float SpMV for a real
// FP32-valued CSR matrix: the caller passes the matrix, x and y as device
// pointers it already owns, and the only scratch the kernel needs -- x split
// into FP32 (hi, lo) pairs -- lives in a fixed array compiled into the library.
//
// Scratch rules:
//   * g_split holds BLQH_NOALLOC_MAX_DIM pairs (8 MiB). Every GPU that loads
//     the library keeps it for the life of the process.
//   * Host code must not pass &g_split to a kernel: on the host that name is a
//     stand-in, not a device address. The first call on each device looks up
//     the array's device address with cudaGetSymbolAddress, with that device
//     current, and caches it; make that first call before any stream capture.
//     The cache is keyed by device number: after a cudaDeviceReset of that
//     device the module may be reloaded elsewhere and the cached address is stale.
//   * All calls share the array and it keeps the last call's contents. Each
//     call overwrites entries [0, dim) before reading them, so nothing needs
//     clearing. Calls that overlap on the GPU (different streams, or different
//     host threads on one device) race on it: order them.
#include <mutex>
#include <string>
#include <vector>

#include "blqh_internal.h"

namespace {

static __device__ __align__(256) float2 g_split[BLQH_NOALLOC_MAX_DIM];

struct DeviceScratch {
  float2* split = nullptr;
  int num_sms = 0;
};
std::mutex g_mu;
std::vector<DeviceScratch> g_dev;

// Device address of g_split (and the SM count) for the current device, looked
// up once per device.
int scratch_for_current_device(DeviceScratch* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(nullptr, BLQH_ERR_CUDA, std::string("blqh_spmv_f32_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return BLQH_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if ((int)g_dev.size() <= dev) g_dev.resize(dev + 1);
  DeviceScratch& d = g_dev[dev];
  if (!d.split) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_split);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || !p) {
      set_error(nullptr, BLQH_ERR_CUDA,
                std::string("blqh_spmv_f32_noalloc: scratch address lookup failed: ") + cudaGetErrorString(e));
      return BLQH_ERR_CUDA;
    }
    d.split = static_cast<float2*>(p);
  }
  *out = d;
  return BLQH_OK;
}

__device__ __forceinline__ void na_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__global__ void k_na_split(const double* __restrict__ x, float2* __restrict__ xs, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float hi = (float)v;
    xs[i] = make_float2(hi, (float)(v - (double)hi));
  }
}

// One warp per row; each product v * (hi + lo) is accumulated as an
// unevaluated FP32 pair (exact product split by FMA, TwoSum for the running sum).
__global__ void __launch_bounds__(256) k_na_spmv(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                                 const float* __restrict__ val, const float2* __restrict__ xs,
                                                 double* __restrict__ y, int64_t dim) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < dim; r += nwarps) {
    const int64_t s = rp[r], e = rp[r + 1];
    float ah = 0.f, al = 0.f;
    for (int64_t k = s + lane; k < e; k += 32) {
      const float v = val[k];
      const float2 x = xs[col[k]];
      const float p = v * x.x;
      const float pe = fmaf(v, x.x, -p);
      float sum, err;
      na_two_sum(ah, p, sum, err);
      ah = sum;
      al += err + fmaf(v, x.y, pe);
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, ah, o), ol = __shfl_xor_sync(0xffffffffu, al, o);
      float sum, err;
      na_two_sum(ah, oh, sum, err);
      ah = sum;
      al = al + ol + err;
    }
    if (lane == 0) y[r] = (double)ah + (double)al;
  }
}

}  // namespace

extern "C" int blqh_spmv_f32_noalloc(const int64_t* row_ptr, const int32_t* col, const float* val, int64_t dim,
                                     const double* x, double* y, void* stream) {
  if (dim < 0 || (dim > 0 && (!row_ptr || !col || !val || !x || !y))) {
    set_error(nullptr, BLQH_ERR_ARG, "blqh_spmv_f32_noalloc: null pointer or negative dim");
    return BLQH_ERR_ARG;
  }
  if (dim > BLQH_NOALLOC_MAX_DIM) {
    set_error(nullptr, BLQH_ERR_ARG,
              "blqh_spmv_f32_noalloc: dim " + std::to_string(dim) + " exceeds the built-in scratch of " +
                  std::to_string(BLQH_NOALLOC_MAX_DIM) + " entries");
    return BLQH_ERR_ARG;
  }
  if (dim == 0) return BLQH_OK;
  DeviceScratch d;
  int rc = scratch_for_current_device(&d);
  if (rc != BLQH_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t blocks = (dim + 255) / 256;
  if (blocks > (int64_t)d.num_sms * 8) blocks = (int64_t)d.num_sms * 8;
  k_na_split<<<(int)blocks, 256, 0, st>>>(x, d.split, dim);
  int64_t sblocks = (dim * 32 + 255) / 256;
  if (sblocks > (int64_t)d.num_sms * 16) sblocks = (int64_t)d.num_sms * 16;
  k_na_spmv<<<(int)sblocks, 256, 0, st>>>(row_ptr, col, val, d.split, y, dim);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(nullptr, BLQH_ERR_CUDA, std::string("blqh_spmv_f32_noalloc: launch: ") + cudaGetErrorString(e));
    return BLQH_ERR_CUDA;
  }
  return BLQH_OK;
}
