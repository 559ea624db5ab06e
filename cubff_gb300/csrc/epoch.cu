// epoch.cu — the fused epoch kernel (gather -> mutate -> run -> split -> count)
// and the soup-init and self-replication kernels, for all 13 languages.
//
// One thread owns one pair.  Its two 64-byte programs are read from HBM with
// 16-byte loads, the 128 per-byte mutation draws of the reference
// (common_language.h:172-180) are applied in registers, and the 128-byte pair
// tape is staged in shared memory in the bank-per-lane layout of common.cuh, so
// the interpreter's data-dependent byte accesses never bank-conflict.  The
// op count is reduced per warp (redux) and added with one atomic per warp, as
// IncreaseInsnCount does (common_language.h:56-63).
#include <algorithm>
#include <atomic>
#include "internal.h"
#include "epoch_body.cuh"

namespace cubff {
namespace {

// InitPrograms (common_language.h:138-155): one thread per 16-byte chunk.
__global__ void init_kernel(uint8_t *soup, uint64_t n, uint64_t key, int zero_init,
                            uint64_t count) {
  const uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= count * 4) return;
  const uint64_t idx = c >> 2;
  const uint64_t base = kTape * n * key + kTape * idx + (c & 3) * 16;
  uint32_t v[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    uint32_t x = 0;
    if (!zero_init) {
#pragma unroll
      for (int b = 0; b < 4; b++)
        x |= (static_cast<uint32_t>(splitmix64(base + 4 * q + b)) & 0xFFu) << (8 * b);
    }
    v[q] = x;
  }
  reinterpret_cast<uint4 *>(soup)[c] = make_uint4(v[0], v[1], v[2], v[3]);
}

// CheckSelfRep (common_language.h:203-277): per program, 13 noise partners
// x (1 + 4) generations, then the byte-stability vote.  One thread per
// program, its working tape in the shared-memory layout, its 13 final tapes
// in thread-local memory.
template <int L>
__global__ void __launch_bounds__(kThreads) selfrep_kernel(const uint8_t *soup,
                                                           uint64_t epoch_key,
                                                           uint64_t n, uint64_t count,
                                                           uint64_t *result) {
  extern __shared__ __align__(16) uint8_t smem[];
  uint8_t *optab = smem + 2 * kGroups * kGroupBytes;
  const uint32_t tid = threadIdx.x;
  if (LangTraits<L>::kNeedsTable)
    for (uint32_t c = tid; c < 256; c += kThreads) optab[c] = op_of(L, c);
  __syncthreads();
  const uint64_t index = uint64_t(blockIdx.x) * kThreads + tid;
  if (index >= count) return;
  const LaneBytes t{smem, lane_base(tid)};
  const LaneBytes stk{smem + kGroups * kGroupBytes, lane_base(tid)};
  constexpr int kIters = 13, kGens = 4;
  uint8_t fin[kIters][kPair];
  const uint8_t *prog = soup + index * kTape;
  const uint64_t local_seed = splitmix64(n * epoch_key + index);
  for (int it = 0; it < kIters; it++) {
    for (int j = 0; j < kTape; j++) {
      t.set(j, prog[j]);
      t.set(kTape + j, static_cast<uint32_t>(
                           splitmix64(local_seed ^ splitmix64(uint64_t(it + 1) * kTape + j))));
    }
    uint32_t raw;
    evaluate<L>(t, stk, optab, &raw);
    for (int g = 0; g < kGens; g++) {
      for (int j = 0; j < kTape; j++) {
        t.set(j, t.get(kTape + j));
        t.set(kTape + j, static_cast<uint32_t>(splitmix64(
                             local_seed ^ splitmix64(uint64_t(it + 1) * kTape + j))));
      }
      evaluate<L>(t, stk, optab, &raw);
    }
    for (int j = 0; j < kPair; j++) fin[it][j] = static_cast<uint8_t>(t.get(j));
  }
  uint64_t res[2] = {0, 0};
  for (int i = 0; i < kPair; i++) {
    for (int x = 0; x < kIters; x++) {
      if (i < kTape && fin[x][i] != prog[i]) continue;
      uint32_t cnt = 1;
      for (int y = x + 1; y < kIters; y++) cnt += fin[x][i] == fin[y][i];
      if (cnt > kIters / 4) {
        res[i / kTape]++;
        break;
      }
    }
  }
  result[index] = res[0] < res[1] ? res[0] : res[1];
}

template <int L>
int launch_epoch_t(const EpochArgs &a, cudaStream_t stream) {
  const uint64_t npairs = a.n / 2;
  if (npairs == 0) return CUBFF_OK;
  const size_t smem = epoch_smem_bytes<L>();
  static std::atomic<bool> attr_set{false};  // per process; setting it twice is harmless
  if (!attr_set.load()) {
    CUBFF_CUDA_TRY(cudaFuncSetAttribute(epoch_kernel<L>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem)));
    attr_set.store(true);
  }
  const uint64_t grid = (npairs + kThreads - 1) / kThreads;
  epoch_kernel<L><<<static_cast<unsigned>(grid), kThreads, smem, stream>>>(a);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

template <int L>
int launch_selfrep_t(const uint8_t *soup, uint64_t epoch_key, uint64_t n,
                     uint64_t count, uint64_t *result, cudaStream_t stream) {
  if (count == 0) return CUBFF_OK;
  const size_t smem = epoch_smem_bytes<L>();
  const uint64_t grid = (count + kThreads - 1) / kThreads;
  selfrep_kernel<L><<<static_cast<unsigned>(grid), kThreads, smem, stream>>>(
      soup, epoch_key, n, count, result);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

template <template <int> class F, typename... Args>
int dispatch_lang(int lang, Args &&...args) {
  switch (lang) {
    case kBff: return F<kBff>::run(args...);
    case kBffNoheads: return F<kBffNoheads>::run(args...);
    case kBffNoheads4bit: return F<kBffNoheads4bit>::run(args...);
    case kBffPerm: return F<kBffPerm>::run(args...);
    case kBff8: return F<kBff8>::run(args...);
    case kBff8Noheads: return F<kBff8Noheads>::run(args...);
    case kBffSelfmove: return F<kBffSelfmove>::run(args...);
    case kForth: return F<kForth>::run(args...);
    case kForthcopy: return F<kForthcopy>::run(args...);
    case kForthtrivial: return F<kForthtrivial>::run(args...);
    case kForthtrivialReset: return F<kForthtrivialReset>::run(args...);
    case kSubleq: return F<kSubleq>::run(args...);
    case kRsubleq4: return F<kRsubleq4>::run(args...);
  }
  return set_error(CUBFF_ENOTFOUND, "unknown language id %d", lang);
}

template <int L>
struct EpochLauncher {
  static int run(const EpochArgs &a, cudaStream_t s) { return launch_epoch_t<L>(a, s); }
};
template <int L>
struct SelfrepLauncher {
  static int run(const uint8_t *soup, uint64_t key, uint64_t n, uint64_t count,
                 uint64_t *result, cudaStream_t s) {
    return launch_selfrep_t<L>(soup, key, n, count, result, s);
  }
};

}  // namespace

int launch_epoch(int lang, const EpochArgs &a, cudaStream_t stream) {
  return dispatch_lang<EpochLauncher>(lang, a, stream);
}

int launch_selfrep(int lang, const uint8_t *soup, uint64_t epoch_key, uint64_t n,
                   uint64_t count, uint64_t *result, cudaStream_t stream) {
  return dispatch_lang<SelfrepLauncher>(lang, soup, epoch_key, n, count, result, stream);
}

int launch_init(uint64_t key, uint64_t n, uint8_t *soup, int zero_init,
                uint64_t count, cudaStream_t stream) {
  if (count == 0) return CUBFF_OK;
  const uint64_t chunks = count * 4;
  const unsigned grid = static_cast<unsigned>((chunks + 255) / 256);
  init_kernel<<<grid, 256, 0, stream>>>(soup, n, key, zero_init, count);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

// Byte histogram of a soup (the statistics of common_language.h:519-533):
// per-block counters in shared memory, added into 256 global counters.
__global__ void histogram_kernel(const uint32_t *words, uint64_t n_words,
                                 unsigned long long *counts) {
  __shared__ uint32_t h[256];
  for (uint32_t c = threadIdx.x; c < 256; c += blockDim.x) h[c] = 0;
  __syncthreads();
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n_words;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t w = words[i];
    atomicAdd(&h[w & 0xFF], 1u);
    atomicAdd(&h[(w >> 8) & 0xFF], 1u);
    atomicAdd(&h[(w >> 16) & 0xFF], 1u);
    atomicAdd(&h[w >> 24], 1u);
  }
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < 256; c += blockDim.x)
    if (h[c]) atomicAdd(&counts[c], static_cast<unsigned long long>(h[c]));
}

int launch_histogram(const uint8_t *soup, uint64_t n_bytes, unsigned long long *counts,
                     cudaStream_t stream) {
  CUBFF_CUDA_TRY(cudaMemsetAsync(counts, 0, 256 * sizeof(unsigned long long), stream));
  const uint64_t words = n_bytes / 4;  // soups are num_programs * 64 bytes
  if (words == 0) return CUBFF_OK;
  const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((words + 255) / 256, 1216));
  histogram_kernel<<<blocks, 256, 0, stream>>>(reinterpret_cast<const uint32_t *>(soup), words,
                                               counts);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

}  // namespace cubff
