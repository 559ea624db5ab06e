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

// Exclusive scan of cnt per epoch segment into start (cnt is then zeroed for
// reuse as the fill cursor), in chunks of kScanChunk counts: one 1024-thread
// block per (chunk, epoch) sums its chunk, then one per (chunk, epoch) adds
// the sums of the epoch's earlier chunks to its own in-chunk scan.
constexpr uint32_t kScanChunk = 4096;

__device__ __forceinline__ uint32_t block_sum_1024(uint32_t v, uint32_t *warp_sums) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = __reduce_add_sync(0xffffffffu, v);
  if (lane == 0) warp_sums[warp] = v;
  __syncthreads();
  uint32_t t = warp_sums[lane];
  t = __reduce_add_sync(0xffffffffu, t);
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(1024) fy_chunk_sums(uint64_t n, uint32_t E, uint32_t chunks,
                                                      const uint32_t *cnt, uint32_t *sums) {
  __shared__ uint32_t warp_sums[32];
  const uint32_t c = blockIdx.x;
  for (uint32_t e = blockIdx.y; e < E; e += gridDim.y) {
    const uint32_t *ce = cnt + uint64_t(e) * n;
    const uint64_t x0 = uint64_t(c) * kScanChunk + threadIdx.x * 4;
    uint32_t v = 0;
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (x0 + q < n) v += ce[x0 + q];
    const uint32_t t = block_sum_1024(v, warp_sums);
    if (threadIdx.x == 0) sums[uint64_t(e) * chunks + c] = t;
  }
}

__global__ void __launch_bounds__(1024) fy_chunk_scan(uint64_t n, uint32_t E, uint32_t chunks,
                                                      uint32_t *cnt, uint32_t *start,
                                                      const uint32_t *sums) {
  __shared__ uint32_t warp_sums[32];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, c = blockIdx.x;
  for (uint32_t e = blockIdx.y; e < E; e += gridDim.y) {
    // The sums of the epoch's chunks before this one.
    uint32_t before = 0;
    for (uint32_t q = tid; q < c; q += 1024) before += sums[uint64_t(e) * chunks + q];
    const uint32_t carry = block_sum_1024(before, warp_sums);
    uint32_t *ce = cnt + uint64_t(e) * n;
    uint32_t *se = start + uint64_t(e) * n;
    const uint64_t x0 = uint64_t(c) * kScanChunk + tid * 4;
    uint32_t v[4], sum = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      v[q] = x0 + q < n ? ce[x0 + q] : 0;
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
      const uint32_t ws = warp_sums[lane];
      uint32_t wi = ws;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, wi, d);
        if (lane >= d) wi += y;
      }
      warp_sums[lane] = wi - ws;  // exclusive prefix of warps
    }
    __syncthreads();
    uint32_t run = carry + warp_sums[warp] + incl - sum;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (x0 + q < n) {
        se[x0 + q] = run;
        ce[x0 + q] = 0;
      }
      run += v[q];
    }
    __syncthreads();  // warp_sums is reused by the next epoch
  }
}

// Exclusive scan of E segments of n counts (cnt -> start, cnt zeroed); sums
// holds E * ceil(n / kScanChunk) words of scratch.
void launch_segment_scan(uint64_t n, uint32_t E, uint32_t *cnt, uint32_t *start, uint32_t *sums,
                         cudaStream_t stream) {
  const uint64_t chunks = (n + kScanChunk - 1) / kScanChunk;
  const dim3 grid(static_cast<unsigned>(chunks), E < 65535u ? E : 65535u);
  fy_chunk_sums<<<grid, 1024, 0, stream>>>(n, E, static_cast<uint32_t>(chunks), cnt, sums);
  fy_chunk_scan<<<grid, 1024, 0, stream>>>(n, E, static_cast<uint32_t>(chunks), cnt, start, sums);
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

// ---------------------------------------------------------------------------
// Pattern (2-D) pairing (common_language.h:435-463) on the device.
//
// The reference, on the host: take the Fisher-Yates order of 0..n-1 (the
// draws of do_shuffle); for each i in that order with a non-empty list,
// propose nb_i = list_i[seed(seed(epoch) ^ seed(i)) % |list_i|]; accept the
// pair (i, nb_i) when neither i nor nb_i is used yet, and mark both.  Then
// the unused programs follow in increasing order.
//
// That is greedy matching in a fixed priority order (the rank of i in the
// order) over one proposal edge per program, and is rebuilt exactly in
// parallel (greedy matching in rounds, Blelloch, Fineman and Shun, SPAA
// 2012): edge e_i is accepted iff no edge of smaller rank that touches i or
// nb_i is accepted.  The edges that can block e_i are e_{nb_i} and every e_j
// with nb_j in {i, nb_i}; each round decides the undecided edges whose
// blockers of smaller rank are all decided (one accepted blocker rejects at
// once).  The smallest-rank undecided edge is always decidable, so rounds
// end; with random ranks a few dozen suffice.  Accepted edges are then
// written in rank order and unused programs in increasing order, both placed
// by prefix sums.
enum : uint8_t { kUndecided = 0, kAccepted = 1, kRejected = 2, kNoEdge = 3 };

// nb[e][i] (or -1 for an empty list), and the in-degree counts for the
// in-lists (cnt[e][v] += 1 for nb = v).
__global__ void pat_propose(uint64_t s0, uint64_t first_epoch, uint64_t n, uint64_t m,
                            const uint32_t *offs, const uint32_t *tgts, int32_t *nb,
                            uint32_t *cnt, uint8_t *status) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n, i = idx - e * n;
  const uint32_t lo = offs[i], len = offs[i + 1] - lo;
  if (len == 0) {
    nb[idx] = -1;
    status[idx] = kNoEdge;
    return;
  }
  const uint64_t ek = seed_from(s0, first_epoch + e);
  const uint32_t v = tgts[lo + seed_from(s0, ek ^ seed_from(s0, i)) % len];
  nb[idx] = static_cast<int32_t>(v);
  status[idx] = kUndecided;
  atomicAdd(&cnt[e * n + v], 1u);
}

// bucket[e][start[v] ..] = the programs j with nb_j = v.
__global__ void pat_fill(uint64_t n, uint64_t m, const int32_t *nb, uint32_t *cnt,
                         const uint32_t *start, uint32_t *bucket) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m || nb[idx] < 0) return;
  const uint64_t e = idx / n, i = idx - e * n;
  const uint64_t g = e * n + static_cast<uint32_t>(nb[idx]);
  bucket[e * n + start[g] + atomicAdd(&cnt[g], 1u)] = static_cast<uint32_t>(i);
}

// One round over the undecided edges (statuses only move from undecided to
// final, so reading a neighbour's status from this same round is safe).
__global__ void pat_round(uint64_t n, uint64_t m, const int32_t *nb, const uint32_t *rank,
                          const uint32_t *start, const uint32_t *len, const uint32_t *bucket,
                          uint8_t *status, uint32_t *undecided) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  if (static_cast<volatile uint8_t *>(status)[idx] != kUndecided) return;
  const uint64_t e = idx / n, i = idx - e * n, base = e * n;
  const volatile uint8_t *st = status + base;
  const uint32_t r = rank[idx];
  const uint32_t b = static_cast<uint32_t>(nb[idx]);
  bool all_decided = true;
  // e_b, the edge proposed by the neighbour.
  if (rank[base + b] < r) {
    const uint8_t x = st[b];
    if (x == kAccepted) {
      status[idx] = kRejected;
      return;
    }
    all_decided &= x != kUndecided;
  }
  // Every e_j with nb_j = i or nb_j = b (e_i itself among the latter).
  for (int side = 0; side < 2; side++) {
    const uint32_t v = side ? b : static_cast<uint32_t>(i);
    const uint32_t s = start[base + v], l = len[base + v];
    for (uint32_t q = 0; q < l; q++) {
      const uint32_t j = bucket[base + s + q];
      if (j == i || rank[base + j] >= r) continue;
      const uint8_t x = st[j];
      if (x == kAccepted) {
        status[idx] = kRejected;
        return;
      }
      all_decided &= x != kUndecided;
    }
  }
  if (all_decided) status[idx] = kAccepted;
  else atomicAdd(&undecided[e], 1u);
}

// used[e][v] for both ends of every accepted edge; flags for the two prefix
// sums: accepted edges by rank, unused programs by id.
__global__ void pat_flags(uint64_t n, uint64_t m, const uint32_t *order, const int32_t *nb,
                          const uint8_t *status, uint8_t *used) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  if (status[idx] == kAccepted) {
    const uint64_t e = idx / n;
    used[idx] = 1;
    used[e * n + static_cast<uint32_t>(nb[idx])] = 1;
  }
}

__global__ void pat_count(uint64_t n, uint64_t m, const uint32_t *order, const uint8_t *status,
                          const uint8_t *used, uint32_t *acc_by_rank, uint32_t *unused_by_id) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n;
  acc_by_rank[idx] = status[e * n + order[idx]] == kAccepted;
  unused_by_id[idx] = used[idx] == 0;
}

// The pairing: accepted edges in rank order (pos from the first scan), then
// the unused programs in id order (pos from the second).  num_indices[e] =
// the number of accepted edges.
__global__ void pat_write(uint64_t n, uint64_t m, const uint32_t *order, const int32_t *nb,
                          const uint8_t *status, const uint8_t *used, const uint32_t *acc_pos,
                          const uint32_t *unused_pos, uint32_t *out, uint64_t *num_indices) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m) return;
  const uint64_t e = idx / n, t = idx - e * n, base = e * n;
  const uint64_t num = acc_pos[base + n - 1] +
                       (status[base + order[base + n - 1]] == kAccepted ? 1 : 0);
  const uint32_t i = order[idx];
  if (status[base + i] == kAccepted) {
    const uint32_t p = acc_pos[idx];
    out[base + 2 * p] = i;
    out[base + 2 * p + 1] = static_cast<uint32_t>(nb[base + i]);
  }
  if (used[idx] == 0) out[base + 2 * num + unused_pos[idx]] = static_cast<uint32_t>(t);
  if (t == 0) num_indices[e] = num;
}

}  // namespace

// Scratch of launch_pattern: the shuffle's own scratch, then order, rank,
// nb, cnt, start, len, bucket, two scan arrays (uint32 each), status and
// used (bytes), and one undecided counter per epoch.
size_t pattern_scratch_bytes(uint64_t n, uint32_t n_epochs) {
  const uint64_t m = n * n_epochs;
  return shuffle_scratch_bytes(n, n_epochs) + 9 * m * sizeof(uint32_t) + 2 * m +
         size_t(n_epochs) * sizeof(uint32_t) + 64;
}

int launch_pattern(uint64_t s0, uint64_t first_epoch, uint32_t E, uint64_t n,
                   const uint32_t *offs, const uint32_t *tgts, uint32_t *out,
                   uint64_t *num_indices, void *scratch, uint32_t *h_undecided,
                   cudaStream_t stream) {
  if (n == 0 || E == 0) return CUBFF_OK;
  const uint64_t m = n * E;
  uint8_t *p = static_cast<uint8_t *>(scratch);
  void *fy = p;
  p += shuffle_scratch_bytes(n, E);
  auto take32 = [&]() {
    uint32_t *a = reinterpret_cast<uint32_t *>(p);
    p += m * sizeof(uint32_t);
    return a;
  };
  uint32_t *order = take32(), *rank = take32();
  int32_t *nb = reinterpret_cast<int32_t *>(take32());
  uint32_t *cnt = take32(), *start = take32(), *len = take32(), *bucket = take32();
  uint32_t *acc = take32(), *unused = take32();
  uint8_t *status = p;
  p += m;
  uint8_t *used = p;
  p += m;
  p = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
  uint32_t *undecided = reinterpret_cast<uint32_t *>(p);
  const unsigned blocks = blocks_for(m, 256);

  CUBFF_TRY(launch_shuffle(s0, first_epoch, E, n, order, fy, stream));
  CUBFF_TRY(launch_inverse(order, E, n, rank, stream));
  CUBFF_CUDA_TRY(cudaMemsetAsync(cnt, 0, m * sizeof(uint32_t), stream));
  CUBFF_CUDA_TRY(cudaMemsetAsync(used, 0, m, stream));
  pat_propose<<<blocks, 256, 0, stream>>>(s0, first_epoch, n, m, offs, tgts, nb, cnt, status);
  // In-degree counts -> lists: len keeps the counts, start their prefix sums.
  CUBFF_CUDA_TRY(cudaMemcpyAsync(len, cnt, m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
  // (also zeroes cnt; the chunk sums go to the shuffle's scratch, free by now)
  launch_segment_scan(n, E, cnt, start, static_cast<uint32_t *>(fy), stream);
  pat_fill<<<blocks, 256, 0, stream>>>(n, m, nb, cnt, start, bucket);
  // Rounds until every edge is decided (checked every 8 rounds).
  for (int checks = 0;; checks++) {
    CUBFF_CUDA_TRY(cudaMemsetAsync(undecided, 0, E * sizeof(uint32_t), stream));
    for (int r = 0; r < 8; r++) {
      if (r == 7) CUBFF_CUDA_TRY(cudaMemsetAsync(undecided, 0, E * sizeof(uint32_t), stream));
      pat_round<<<blocks, 256, 0, stream>>>(n, m, nb, rank, start, len, bucket, status, undecided);
    }
    CUBFF_CUDA_TRY(cudaMemcpyAsync(h_undecided, undecided, E * sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, stream));
    CUBFF_CUDA_TRY(cudaStreamSynchronize(stream));
    uint64_t left = 0;
    for (uint32_t e = 0; e < E; e++) left += h_undecided[e];
    if (left == 0) break;
    if (checks > static_cast<int>(n)) return set_error(CUBFF_EDEVICE, "pattern pairing did not converge");
  }
  pat_flags<<<blocks, 256, 0, stream>>>(n, m, order, nb, status, used);
  pat_count<<<blocks, 256, 0, stream>>>(n, m, order, status, used, acc, unused);
  // Exclusive prefix sums per epoch (each scan reads its counts, writes the
  // sums, zeroes the counts).
  launch_segment_scan(n, E, acc, start, static_cast<uint32_t *>(fy), stream);
  launch_segment_scan(n, E, unused, len, static_cast<uint32_t *>(fy), stream);
  pat_write<<<blocks, 256, 0, stream>>>(n, m, order, nb, status, used, start, len, out, num_indices);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

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
  // The chunk sums live in nxt until fy_link writes it.
  launch_segment_scan(n, E, b.cnt, b.start, reinterpret_cast<uint32_t *>(b.nxt), stream);
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
