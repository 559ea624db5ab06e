// pairing.cu — the reference's host-side pairings, computed on the device for
// many epochs per launch.
//
// Fisher-Yates (do_shuffle, common_language.h:418-424) is serial on the host
// in the reference: s = identity; for i = n-1 .. 0: j_i = SplitMix64(seed(
// epoch*n + i)) % (i+1); swap(s[i], s[j_i]).  Its result is rebuilt exactly
// and in parallel from the draws j_i:
//   * step i writes s[i] for good (later steps touch only indices < i), taking
//     the value that position j_i holds just before step i;
//   * the last write into position p before step i is made by
//     next(i) = min{k > i : j_k = j_i}, which moves V(next(i)) there, where
//     V(k) is the value at position k just before step k;
//   * V(k) = V(parent(k)) with parent(k) = min{k' > k : j_k' = k}, and
//     V(k) = k when no such k' exists (the position was never written);
//   * so s[i] = V(next(i)) if next(i) exists, else j_i.
// Draws are grouped by value with a counting sort (count, scan, fill); next()
// and parent() are scans of the (small) groups; V follows parent() chains,
// which strictly increase and so end.
#include <mutex>

#include "internal.h"
#include "common.cuh"

namespace cubff {
namespace {

struct FyBufs {
  uint32_t *j, *cnt, *start, *bucket;
  int32_t *nxt, *par;
};

FyBufs fy_bufs(void *scratch, uint64_t n, uint32_t E) {
  const uint64_t m = n * E;
  uint32_t *base = static_cast<uint32_t *>(scratch);
  FyBufs b;
  b.j = base;
  b.cnt = base + m;
  b.start = base + 2 * m;
  b.bucket = base + 3 * m;
  b.nxt = reinterpret_cast<int32_t *>(base + 4 * m);
  b.par = reinterpret_cast<int32_t *>(base + 5 * m);
  return b;
}

__global__ void fy_draw(uint64_t s0, uint64_t first_epoch, uint64_t n, uint64_t m,
                        uint32_t *j, uint32_t *cnt) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n, i = idx - e * n;
  const uint64_t key = seed_from(s0, (first_epoch + e) * n + i);
  const uint32_t ji = static_cast<uint32_t>(splitmix64(key) % (i + 1));
  j[idx] = ji;
  atomicAdd(&cnt[e * n + ji], 1u);
}

// Exclusive scan of cnt per epoch segment into start; cnt is then zeroed for
// reuse as the fill cursor.  One 1024-thread block per epoch.
__global__ void __launch_bounds__(1024) fy_scan(uint64_t n, uint32_t *cnt, uint32_t *start) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t carry_s;
  const uint64_t off = uint64_t(blockIdx.x) * n;
  uint32_t *c = cnt + off;
  uint32_t *s = start + off;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) carry_s = 0;
  __syncthreads();
  for (uint64_t base = 0; base < n; base += 4096) {
    uint32_t v[4];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint64_t x = base + tid * 4 + q;
      v[q] = x < n ? c[x] : 0;
      sum += v[q];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t ws = warp_sums[lane];
      uint32_t wi = ws;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, wi, d);
        if (lane >= d) wi += y;
      }
      warp_sums[lane] = wi - ws;  // exclusive prefix of warps
    }
    __syncthreads();
    uint32_t run = carry_s + warp_sums[warp] + incl - sum;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint64_t x = base + tid * 4 + q;
      if (x < n) {
        s[x] = run;
        c[x] = 0;
      }
      run += v[q];
    }
    __syncthreads();
    if (tid == 1023) carry_s = run;
    __syncthreads();
  }
}

__global__ void fy_fill(uint64_t n, uint64_t m, const uint32_t *j, uint32_t *cnt,
                        const uint32_t *start, uint32_t *bucket) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n, i = idx - e * n;
  const uint64_t g = e * n + j[idx];
  const uint32_t pos = atomicAdd(&cnt[g], 1u);
  bucket[e * n + start[g] + pos] = static_cast<uint32_t>(i);
}

// nxt[i] = min{k > i : j_k = j_i}, par[i] = min{k > i : j_k = i} (or -1).
__global__ void fy_link(uint64_t n, uint64_t m, const uint32_t *j, const uint32_t *cnt,
                        const uint32_t *start, const uint32_t *bucket, int32_t *nxt,
                        int32_t *par) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n, i = idx - e * n;
  const uint32_t *bk = bucket + e * n;
  auto min_above = [&](uint64_t g) -> int32_t {
    const uint32_t b0 = start[e * n + g], len = cnt[e * n + g];
    uint32_t best = 0xffffffffu;
    for (uint32_t q = 0; q < len; q++) {
      const uint32_t k = bk[b0 + q];
      if (k > i && k < best) best = k;
    }
    return best == 0xffffffffu ? -1 : static_cast<int32_t>(best);
  };
  nxt[idx] = min_above(j[idx]);
  par[idx] = min_above(i);
}

__global__ void fy_resolve(uint64_t n, uint64_t m, const uint32_t *j, const int32_t *nxt,
                           const int32_t *par, uint32_t *out) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n;
  const int32_t *pe = par + e * n;
  int32_t v = nxt[idx];
  if (v < 0) {
    out[idx] = j[idx];
    return;
  }
  while (pe[v] >= 0) v = pe[v];  // strictly increasing, so it ends
  out[idx] = static_cast<uint32_t>(v);
}

// fixed_shuffle (common_language.h:468-474).
__global__ void fixed_kernel(uint64_t first_epoch, uint64_t n, uint64_t m, uint32_t *out) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = first_epoch + idx / n, i = idx % n;
  const uint64_t max_pow2 = 31 - __clz(static_cast<unsigned>(n));
  const uint64_t offset = (1ull << (e % max_pow2 + 1)) - 1;
  out[idx] = static_cast<uint32_t>(((i * offset) % n) ^ (e & 1));
}

// permute_programs == false (common_language.h:478-486).
__global__ void cyclic_kernel(uint64_t first_epoch, uint64_t n, uint64_t m, uint32_t *out) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = first_epoch + idx / n, i = idx % n;
  out[idx] = (e % 2 == 1) ? static_cast<uint32_t>(i)
                          : static_cast<uint32_t>(i == 0 ? n - 1 : i - 1);
}

// inv[e][perm[e][i]] = i: the position of each program in an epoch's shuffle.
__global__ void inverse_kernel(const uint32_t *perm, uint64_t n, uint64_t m, uint32_t *inv) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n;
  inv[e * n + perm[idx]] = static_cast<uint32_t>(idx - e * n);
}

unsigned blocks_for(uint64_t m, unsigned t) { return static_cast<unsigned>((m + t - 1) / t); }

}  // namespace

// Six uint32 arrays of n * n_epochs entries; SIZE_MAX when that does not fit
// in size_t (so no scratch size can pass a check against it).
size_t shuffle_scratch_bytes(uint64_t n, uint32_t n_epochs) {
  constexpr uint64_t kPerDraw = 6 * sizeof(uint32_t);
  if (n_epochs != 0 && n > (SIZE_MAX / kPerDraw) / n_epochs) return SIZE_MAX;
  return size_t(kPerDraw) * n * n_epochs;
}

int launch_shuffle(uint64_t s0, uint64_t first_epoch, uint32_t E, uint64_t n,
                   uint32_t *out, void *scratch, cudaStream_t stream) {
  if (n == 0 || E == 0) return CUBFF_OK;
  const uint64_t m = n * E;
  FyBufs b = fy_bufs(scratch, n, E);
  CUBFF_CUDA_TRY(cudaMemsetAsync(b.cnt, 0, m * sizeof(uint32_t), stream));
  fy_draw<<<blocks_for(m, 256), 256, 0, stream>>>(s0, first_epoch, n, m, b.j, b.cnt);
  fy_scan<<<E, 1024, 0, stream>>>(n, b.cnt, b.start);
  fy_fill<<<blocks_for(m, 256), 256, 0, stream>>>(n, m, b.j, b.cnt, b.start, b.bucket);
  fy_link<<<blocks_for(m, 256), 256, 0, stream>>>(n, m, b.j, b.cnt, b.start, b.bucket,
                                                  b.nxt, b.par);
  fy_resolve<<<blocks_for(m, 256), 256, 0, stream>>>(n, m, b.j, b.nxt, b.par, out);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

int launch_inverse(const uint32_t *perm, uint32_t E, uint64_t n, uint32_t *inv,
                   cudaStream_t stream) {
  const uint64_t m = n * E;
  if (m == 0) return CUBFF_OK;
  inverse_kernel<<<blocks_for(m, 256), 256, 0, stream>>>(perm, n, m, inv);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

int launch_fixed(uint64_t first_epoch, uint32_t E, uint64_t n, uint32_t *out,
                 cudaStream_t stream) {
  const uint64_t m = n * E;
  if (m == 0) return CUBFF_OK;
  fixed_kernel<<<blocks_for(m, 256), 256, 0, stream>>>(first_epoch, n, m, out);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

int launch_cyclic(uint64_t first_epoch, uint32_t E, uint64_t n, uint32_t *out,
                  cudaStream_t stream) {
  const uint64_t m = n * E;
  if (m == 0) return CUBFF_OK;
  cyclic_kernel<<<blocks_for(m, 256), 256, 0, stream>>>(first_epoch, n, m, out);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

}  // namespace cubff

// ---------------------------------------------------------------------------
// Allocation-free Fisher-Yates pairing.
//
// For callers that cannot allocate device memory themselves: a host
// application that owns the device allocator (it reserves the GPU's memory up
// front and forbids other code to call cudaMalloc), or a code path where the
// implicit device-wide synchronisation of cudaMalloc / cudaFree is not
// acceptable.  Such a caller passes only its output buffer; the scratch of the
// pairing kernels is a fixed array in this library's device memory.
//
// Limits and behaviour:
//  * The scratch holds kNoAllocMaxDraws draws (num_programs * n_epochs), i.e.
//    6 MiB, reserved on every GPU that loads this library until the process
//    exits.  Larger requests are rejected with CUBFF_EINVAL.
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that
//    first call before any stream capture.  cudaDeviceReset (or anything else
//    that destroys the device's primary context) invalidates the cached
//    address: do not call this entry point on that device afterwards.
//  * All calls share the one array.  The counts the kernels accumulate are
//    cleared at the start of every call; everything else is overwritten.
//    Calls whose work overlaps on the GPU (different streams, or different
//    host threads without ordering) race on the array: order them.
namespace cubff {
namespace {

constexpr uint64_t kNoAllocMaxDraws = uint64_t(1) << 18;
static __device__ __align__(256) uint32_t g_noalloc_scratch[6 * kNoAllocMaxDraws];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[64] = {nullptr};

}  // namespace

}  // namespace cubff

extern "C" int cubff_shuffle_indices_noalloc(uint64_t params_seed, uint64_t first_epoch,
                                             uint32_t n_epochs, uint64_t num_programs,
                                             uint32_t *d_out, void *stream) {
  using namespace cubff;
  if (!d_out || num_programs == 0 || n_epochs == 0)
    return set_error(CUBFF_EINVAL, "shuffle_indices_noalloc: bad arguments");
  // Tested by division: the product itself could wrap.
  if (num_programs > kNoAllocMaxDraws || n_epochs > kNoAllocMaxDraws / num_programs)
    return set_error(CUBFF_EINVAL,
                     "shuffle_indices_noalloc: num_programs %llu x n_epochs %u exceeds the "
                     "built-in scratch limit of %llu draws",
                     static_cast<unsigned long long>(num_programs), n_epochs,
                     static_cast<unsigned long long>(kNoAllocMaxDraws));
  int dev = 0;
  CUBFF_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(CUBFF_EINVAL, "shuffle_indices_noalloc: device %d", dev);
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void *p = nullptr;
      cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (err != cudaSuccess || !p)
        return set_error(CUBFF_EDEVICE, "shuffle_indices_noalloc: cudaGetSymbolAddress: %s",
                         cudaGetErrorString(err));
      g_noalloc_addr[dev] = p;
    }
    scratch = g_noalloc_addr[dev];
  }
  return launch_shuffle(splitmix64(params_seed), first_epoch, n_epochs, num_programs, d_out,
                        scratch, static_cast<cudaStream_t>(stream));
}
