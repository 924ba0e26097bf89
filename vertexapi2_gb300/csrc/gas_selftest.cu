// gas_selftest_bounded_waits (gas_gb300.h): runs the engine's two device
// wait primitives against partners that never arrive and reports what the
// host sees -- the failure path of a stalled round, exercised without any
// fault: each wait gives up at its spin limit, sets GAS_DEVERR_TIMEOUT and
// returns, and the kernel ends normally.
#include <cuda_runtime.h>

#include <chrono>

#include "gas_gb300.h"
#include "gas_gb300/detail/persistent.cuh"
#include "gas_internal.h"

using gas::internal::cuda_fail;
using gas::internal::fail;

namespace {

// Cooperative launch of two blocks; only block 0 enters the grid barrier,
// so its partner never arrives.
__global__ void stalled_barrier_kernel(unsigned *bar, unsigned *err, int32_t *result) {
  if (blockIdx.x != 0) return;
  const bool ok = gas::detail::grid_barrier(bar, err);
  if (threadIdx.x == 0) *result = ok ? 1 : 0;
}

// A look-back wait on a tile flag that no tile publishes.
__global__ void stalled_lookback_kernel(const unsigned *flag, unsigned *err, int32_t *result) {
  if (threadIdx.x != 0) return;
  unsigned act = 0u;
  const bool ok = gas::detail::wait_epoch(flag, 7u, err, &act);
  *result = ok ? 1 : 0;
}

gas_status to_status(unsigned err, int32_t result) {
  if (result == 0 && (err & GAS_DEVERR_TIMEOUT)) return GAS_ERR_TIMEOUT;
  return result == 1 ? GAS_OK : GAS_ERR_CUDA;
}

}  // namespace

extern "C" gas_status gas_selftest_bounded_waits(int32_t device, gas_status *barrierStatus,
                                                 gas_status *lookbackStatus, float *seconds) {
  if (!barrierStatus || !lookbackStatus) return fail(GAS_ERR_INVALID, "null argument");
  if (!gas_device_supported(device)) return fail(GAS_ERR_NO_DEVICE, "device %d is not sm_103", device);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  unsigned *mem = nullptr;  // bar[2] | err | flag | result[2]
  cudaError_t e = cudaMalloc(&mem, 8 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(mem, 0, 8 * sizeof(unsigned));
  const auto t0 = std::chrono::steady_clock::now();
  if (e == cudaSuccess) {
    unsigned *bar = mem, *err = mem + 2;
    int32_t *res = reinterpret_cast<int32_t *>(mem + 4);
    void *args[] = {&bar, &err, &res};
    e = cudaLaunchCooperativeKernel((const void *)stalled_barrier_kernel, dim3(2), dim3(32), args,
                                    0, nullptr);
  }
  unsigned host[8] = {0};
  if (e == cudaSuccess) e = cudaMemcpy(host, mem, sizeof(host), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) *barrierStatus = to_status(host[2], (int32_t)host[4]);
  if (e == cudaSuccess) e = cudaMemset(mem + 2, 0, sizeof(unsigned));
  if (e == cudaSuccess) {
    stalled_lookback_kernel<<<1, 32>>>(mem + 3, mem + 2, reinterpret_cast<int32_t *>(mem + 5));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host, mem, sizeof(host), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) *lookbackStatus = to_status(host[2], (int32_t)host[5]);
  const auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<float>(t1 - t0).count();
  if (mem) cudaFree(mem);
  if (prev >= 0) cudaSetDevice(prev);
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "bounded-wait self test");
}
