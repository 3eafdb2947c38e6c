// Self-test of the bounded mbarrier wait that every pipelined kernel uses
// (msx_tma.cuh): one CTA waits on a barrier that receives no arrival unless
// asked to, with a short limit, and reports through an error word exactly as
// the passes do.  It exercises the timeout path without faulting or hanging
// the GPU.
#include "msx.h"
#include "msx_internal.h"
#include "msx_tma.cuh"

namespace {

__global__ void wait_selftest_kernel(int arrive, long long limit, int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    msx::mbar_init(&bar, 1);
    msx::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (arrive) msx::mbar_arrive(&bar);
    if (!msx::mbar_wait_bounded(&bar, 0, limit)) atomicOr(err, 1);
  }
}

}  // namespace

extern "C" {

int msx_selftest_wait(int arrive, int limit_log2, void* stream) {
  if (limit_log2 < 10 || limit_log2 > 31) {
    msx::set_last_error("msx_selftest_wait: limit_log2 must be in [10, 31]");
    return MSX_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int* err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
    msx::set_last_error("msx_selftest_wait: allocation failed");
    return MSX_ERR_ALLOC;
  }
  int h = 0;
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e == cudaSuccess) {
    wait_selftest_kernel<<<1, 32, 0, st>>>(arrive, 1LL << limit_log2, err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(err);
  if (e != cudaSuccess) {
    msx::set_last_error(cudaGetErrorString(e));
    return MSX_ERR_CUDA;
  }
  if (h) {
    msx::set_last_error("msx_selftest_wait: the bounded wait ran out (as asked)");
    return MSX_ERR_TIMEOUT;
  }
  return MSX_OK;
}

}  // extern "C"
