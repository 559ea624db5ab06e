// batch.cu — many independent soups (uneven size, language, mutation rate)
// advanced together: one persistent launch per epoch covers every pair of
// every soup.  A descriptor per soup (EpochArgs + language + first virtual
// CTA) lets each CTA find its soup by binary search over the CTA prefix; the
// language switch is uniform per CTA, so there is no divergence from mixing
// languages.
#include <algorithm>
#include <vector>

#include "engine_impl.h"
#include "epoch_body.cuh"

namespace cubff {

struct BatchDesc {
  EpochArgs a;
  int lang;
  uint32_t block_begin;  // first virtual CTA of this soup
};

namespace {

__global__ void __launch_bounds__(kThreads)
    batch_epoch_kernel(const BatchDesc *__restrict__ descs, int n_soups, uint32_t total_blocks) {
  extern __shared__ __align__(16) uint8_t smem[];
  for (uint32_t vb = blockIdx.x; vb < total_blocks; vb += gridDim.x) {
    int lo = 0, hi = n_soups - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (descs[mid].block_begin <= vb) lo = mid; else hi = mid - 1;
    }
    const EpochArgs a = descs[lo].a;
    const uint64_t blk = vb - descs[lo].block_begin;
    switch (descs[lo].lang) {
      case kBff: epoch_cta<kBff>(a, blk, smem); break;
      case kBffNoheads: epoch_cta<kBffNoheads>(a, blk, smem); break;
      case kBffNoheads4bit: epoch_cta<kBffNoheads4bit>(a, blk, smem); break;
      case kBffPerm: epoch_cta<kBffPerm>(a, blk, smem); break;
      case kBff8: epoch_cta<kBff8>(a, blk, smem); break;
      case kBff8Noheads: epoch_cta<kBff8Noheads>(a, blk, smem); break;
      case kBffSelfmove: epoch_cta<kBffSelfmove>(a, blk, smem); break;
      case kForth: epoch_cta<kForth>(a, blk, smem); break;
      case kForthcopy: epoch_cta<kForthcopy>(a, blk, smem); break;
      case kForthtrivial: epoch_cta<kForthtrivial>(a, blk, smem); break;
      case kForthtrivialReset: epoch_cta<kForthtrivialReset>(a, blk, smem); break;
      case kSubleq: epoch_cta<kSubleq>(a, blk, smem); break;
      default: epoch_cta<kRsubleq4>(a, blk, smem); break;
    }
    __syncthreads();  // shared memory is reused by the next virtual CTA
  }
}

}  // namespace

int launch_batch_epoch(const BatchDesc *d_descs, int n_soups, uint32_t total_blocks,
                       int device, cudaStream_t stream) {
  static int max_grid[64] = {0};
  int &g = max_grid[device & 63];
  if (g == 0) {
    CUBFF_CUDA_TRY(cudaFuncSetAttribute(batch_epoch_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(kMaxEpochSmem)));
    int per_sm = 0, sms = 0;
    CUBFF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_epoch_kernel,
                                                                 kThreads, kMaxEpochSmem));
    CUBFF_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    g = std::max(1, per_sm) * sms;
  }
  const uint32_t grid = std::min<uint32_t>(total_blocks, static_cast<uint32_t>(g));
  batch_epoch_kernel<<<grid, kThreads, kMaxEpochSmem, stream>>>(d_descs, n_soups, total_blocks);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

}  // namespace cubff

using namespace cubff;

int cubff_engine::reserve_batch(size_t n_desc) {
  if (n_desc <= desc_cap) return CUBFF_OK;
  release_batch();
  CUBFF_CUDA_TRY(cudaMalloc(&d_desc, n_desc * sizeof(BatchDesc)));
  CUBFF_CUDA_TRY(cudaMallocHost(&h_desc, n_desc * sizeof(BatchDesc)));
  CUBFF_CUDA_TRY(cudaMalloc(&d_bcnt, n_desc * 2 * sizeof(unsigned long long)));
  CUBFF_CUDA_TRY(cudaMallocHost(&h_bcnt, n_desc * 2 * sizeof(unsigned long long)));
  desc_cap = n_desc;
  return CUBFF_OK;
}

void cubff_engine::release_batch() {
  if (d_desc) cudaFree(d_desc);
  if (h_desc) cudaFreeHost(h_desc);
  if (d_bcnt) cudaFree(d_bcnt);
  if (h_bcnt) cudaFreeHost(h_bcnt);
  d_desc = h_desc = nullptr;
  d_bcnt = h_bcnt = nullptr;
  desc_cap = 0;
}

extern "C" int cubff_batch_run(cubff_engine *eng, cubff_soup **soups, int n_soups,
                               uint64_t n_epochs, uint64_t *ops) {
  if (!eng || !soups || n_soups <= 0 || (!ops && n_epochs))
    return set_error(CUBFF_EINVAL, "batch_run: bad arguments");
  for (int s = 0; s < n_soups; s++) {
    if (!soups[s] || soups[s]->eng != eng)
      return set_error(CUBFF_EINVAL, "batch_run: soup %d is null or on another engine", s);
    if (soups[s]->p.pairing == CUBFF_PAIR_PATTERN && soups[s]->pat_offs.empty())
      return set_error(CUBFF_EINVAL, "batch_run: soup %d needs its interaction lists", s);
    for (int t = 0; t < s; t++)
      if (soups[t] == soups[s]) return set_error(CUBFF_EINVAL, "batch_run: soup %d repeated", s);
  }
  CUBFF_CUDA_TRY(cudaSetDevice(eng->device));
  cudaStream_t st = eng->stream;
  for (int s = 0; s < n_soups; s++) {
    CUBFF_TRY(soups[s]->ensure_buffers());
    if (soups[s]->pending_reset) {
      CUBFF_TRY(soups[s]->apply_reset());
      soups[s]->pending_reset = false;
    }
  }
  std::vector<uint32_t> block_begin(n_soups);
  uint64_t total = 0;
  for (int s = 0; s < n_soups; s++) {
    block_begin[s] = static_cast<uint32_t>(total);
    total += (soups[s]->p.num_programs / 2 + kThreads - 1) / kThreads;
  }
  if (total > 0xffffffffull) return set_error(CUBFF_EINVAL, "batch_run: too many pairs");

  const uint32_t chunk_max = static_cast<uint32_t>(std::min<uint64_t>(n_epochs, 1024));
  CUBFF_TRY(eng->reserve_batch(size_t(chunk_max) * n_soups));
  BatchDesc *hd = static_cast<BatchDesc *>(eng->h_desc);
  BatchDesc *dd = static_cast<BatchDesc *>(eng->d_desc);
  unsigned long long *dc = eng->d_bcnt, *hc = eng->h_bcnt;

  uint64_t done = 0;
  while (done < n_epochs) {
    const uint32_t chunk = static_cast<uint32_t>(std::min<uint64_t>(chunk_max, n_epochs - done));
    CUBFF_CUDA_TRY(cudaMemsetAsync(dc, 0, size_t(2) * chunk * n_soups * sizeof(unsigned long long), st));
    for (uint32_t c = 0; c < chunk; c++) {
      BatchDesc *row = hd + size_t(c) * n_soups;
      for (int s = 0; s < n_soups; s++) {
        cubff_soup *sp = soups[s];
        const uint64_t e = sp->epoch + done + c;
        if (sp->perm_count == 0 || e < sp->perm_first || e >= sp->perm_first + sp->perm_count) {
          const uint64_t remaining = n_epochs - done - c;
          CUBFF_TRY(sp->fill_pairing(e, static_cast<uint32_t>(std::min<uint64_t>(sp->batch, remaining))));
        }
        const uint64_t slot = e - sp->perm_first;
        const uint64_t n = sp->p.num_programs;
        EpochArgs &a = row[s].a;
        a.soup = sp->d_soup;
        a.perm = sp->d_perm + slot * n;
        a.n = n;
        a.num_indices = n / 2;
        a.d_num_indices = sp->p.pairing == CUBFF_PAIR_PATTERN ? sp->d_num_indices + slot : nullptr;
        a.epoch_key = seed_from(sp->s0, e);
        a.mutation_prob = sp->p.mutation_prob;
        a.ops = dc + (size_t(c) * n_soups + s) * 2;
        a.raw = a.ops + 1;
        row[s].lang = sp->p.lang;
        row[s].block_begin = block_begin[s];
      }
      CUBFF_CUDA_TRY(cudaMemcpyAsync(dd + size_t(c) * n_soups, row, sizeof(BatchDesc) * n_soups,
                                     cudaMemcpyHostToDevice, st));
      CUBFF_TRY(launch_batch_epoch(dd + size_t(c) * n_soups, n_soups, static_cast<uint32_t>(total),
                                   eng->device, st));
      for (int s = 0; s < n_soups; s++) {
        cubff_soup *sp = soups[s];
        const uint64_t e = sp->epoch + done + c;
        if (sp->p.reset_interval && e % sp->p.reset_interval == 0) {
          if (done + c + 1 == n_epochs) sp->pending_reset = true;
          else CUBFF_TRY(sp->apply_reset());
        }
      }
    }
    CUBFF_CUDA_TRY(cudaMemcpyAsync(hc, dc, size_t(2) * chunk * n_soups * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, st));
    CUBFF_CUDA_TRY(cudaStreamSynchronize(st));
    for (uint32_t c = 0; c < chunk; c++)
      for (int s = 0; s < n_soups; s++) ops[size_t(s) * n_epochs + done + c] = hc[(size_t(c) * n_soups + s) * 2];
    done += chunk;
  }
  for (int s = 0; s < n_soups; s++) soups[s]->epoch += n_epochs;
  return CUBFF_OK;
}
