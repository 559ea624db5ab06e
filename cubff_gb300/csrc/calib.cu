// calib.cu — measured integer-issue rate of the device (the denominator of
// the epoch step's roofline, and a reference point for the launch-shape
// tuner).
//
// The interpreters are integer code: shared-memory loads, adds, logic, shifts,
// compares and selects.  Their roofline is the rate at which the SMs retire
// 32-bit integer instructions per lane.  Two chains of known instruction
// counts measure it:
//   * alu:   x += y; y ^= x;                       (2 instructions)
//   * mixed: x += y; y ^= x; z = z * K + x;        (3 instructions, the
//            multiply-add on the other integer-capable pipe)
// Each thread runs 8 independent copies of the chain (latency hidden by the
// copies and by 32 resident warps per SM).  An add followed by an xor of its
// result cannot be fused into one instruction, so the source counts are the
// instruction counts.  The result is lane-instructions per second (one lane
// retiring one integer instruction counts 1).
#include "internal.h"

namespace cubff {
namespace {

constexpr int kChains = 8;

template <bool kMixed>
__global__ void __launch_bounds__(256) int_issue_kernel(uint32_t iters, uint32_t seed,
                                                        uint32_t *sink) {
  uint32_t x[kChains], y[kChains], z[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) {
    x[k] = threadIdx.x * (k + 1) + seed;
    y[k] = blockIdx.x + k * 0x9e3779b9u;
    z[k] = seed ^ k;
  }
  for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) {
      x[k] += y[k];
      y[k] ^= x[k];
      if (kMixed) z[k] = z[k] * 0x9e3779b1u + x[k];
    }
  }
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) r ^= x[k] + y[k] + z[k];
  if (r == seed) sink[0] = r;  // keeps every chain live
}

template <bool kMixed>
int time_chain(int sms, uint32_t iters, uint32_t *sink, cudaStream_t st, double *out) {
  const unsigned blocks = static_cast<unsigned>(sms) * 8;  // 8 x 256 threads per SM
  int_issue_kernel<kMixed><<<blocks, 256, 0, st>>>(iters / 16, 1, sink);  // warm-up
  cudaEvent_t a, b;
  CUBFF_CUDA_TRY(cudaEventCreate(&a));
  CUBFF_CUDA_TRY(cudaEventCreate(&b));
  CUBFF_CUDA_TRY(cudaEventRecord(a, st));
  int_issue_kernel<kMixed><<<blocks, 256, 0, st>>>(iters, 1, sink);
  CUBFF_CUDA_TRY(cudaEventRecord(b, st));
  CUBFF_CUDA_TRY(cudaEventSynchronize(b));
  float ms = 0;
  CUBFF_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CUBFF_CUDA_TRY(cudaGetLastError());
  const double instr = double(blocks) * 256 * iters * kChains * (kMixed ? 3 : 2);
  *out = instr / (ms * 1e-3);
  return CUBFF_OK;
}

}  // namespace
}  // namespace cubff

extern "C" int cubff_measure_int_issue(int device, double *alu_per_s, double *mixed_per_s) {
  using namespace cubff;
  if (!alu_per_s || !mixed_per_s) return set_error(CUBFF_EINVAL, "measure_int_issue: null output");
  CUBFF_CUDA_TRY(cudaSetDevice(device));
  int sms = 0;
  CUBFF_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  uint32_t *sink = nullptr;
  CUBFF_CUDA_TRY(cudaMalloc(&sink, sizeof(uint32_t)));
  cudaStream_t st = nullptr;
  cudaError_t err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  int status = err == cudaSuccess ? CUBFF_OK
                                  : set_error(CUBFF_EDEVICE, "cudaStreamCreate: %s",
                                              cudaGetErrorString(err));
  // ~10-40 ms per timed launch on a GB300.
  if (status == CUBFF_OK) status = time_chain<false>(sms, 1u << 17, sink, st, alu_per_s);
  if (status == CUBFF_OK) status = time_chain<true>(sms, 1u << 17, sink, st, mixed_per_s);
  if (st) cudaStreamDestroy(st);
  cudaFree(sink);
  return status;
}
