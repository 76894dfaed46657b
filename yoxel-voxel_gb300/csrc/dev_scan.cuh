// dev_scan.cuh - device helpers shared by the scene builders: stream-ordered
// scratch buffers, grid sizing and an exclusive scan of uint32 counts.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "yv_kernels.h"

namespace yv {
namespace {

constexpr int kScanBlock = 1024;  // elements per block of the scan (256 x 4)

// ---- exclusive scan of uint32 counts (blocks of 1024, recursive sums) ----
__global__ void scan_block_kernel(const uint32_t* in, uint32_t* out, uint32_t* sums, uint32_t n) {
  __shared__ uint32_t warp_tot[8];
  const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * 4;
  uint32_t v[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = base + k < n ? in[base + k] : 0u;
  const uint32_t t = v[0] + v[1] + v[2] + v[3];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t inc = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= (uint32_t)o) inc += u;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  uint32_t wbase = 0;
  for (uint32_t w = 0; w < warp; ++w) wbase += warp_tot[w];
  uint32_t run = wbase + inc - t;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == blockDim.x - 1) {
    uint32_t tot = 0;
    for (int w = 0; w < 8; ++w) tot += warp_tot[w];
    sums[blockIdx.x] = tot;
  }
}

__global__ void scan_add_kernel(uint32_t* out, const uint32_t* offs, uint32_t n) {
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x * 4;
  const uint32_t add = offs[blockIdx.x];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (i + k < n) out[i + k] += add;
}

// Device buffers released on scope exit (stream-ordered).
struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  cudaError_t alloc(size_t bytes, cudaStream_t st) {
    s = st;
    return scratch_alloc(&p, bytes ? bytes : 16, st);
  }
  ~DevBuf() { scratch_free(p, s); }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

int grid_for(uint64_t work) {
  const uint64_t b = (work + 255) / 256;
  const uint64_t cap = (uint64_t)device_sm_count() * 16;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// out[i] = sum of in[0..i); *total = sum of all (read back with a stream
// sync), or total = NULL when the caller knows it (no sync).
cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total,
                           cudaStream_t s) {
  if (n == 0) {
    if (total) *total = 0;
    return cudaSuccess;
  }
  const uint32_t blocks = (n + kScanBlock - 1) / kScanBlock;
  DevBuf sums, offs;
  cudaError_t e = sums.alloc((size_t)blocks * 4, s);
  if (e == cudaSuccess) e = offs.alloc((size_t)blocks * 4, s);
  if (e != cudaSuccess) return e;
  scan_block_kernel<<<blocks, 256, 0, s>>>(in, out, sums.as<uint32_t>(), n);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (blocks > 1) {
    e = exclusive_scan(sums.as<uint32_t>(), offs.as<uint32_t>(), blocks, total, s);
    if (e != cudaSuccess) return e;
    scan_add_kernel<<<blocks, 256, 0, s>>>(out, offs.as<uint32_t>(), n);
    return cudaGetLastError();
  }
  // one block: its sum is the total
  if (!total) return cudaSuccess;
  e = cudaMemcpyAsync(total, sums.as<uint32_t>(), 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace
}  // namespace yv
