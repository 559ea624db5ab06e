// pipeline.cu — epochs of one soup run as a dataflow pipeline instead of one
// launch per epoch.
//
// Pair k of epoch e reads programs s_e[2k], s_e[2k+1] as epoch e-1 left them
// and writes them back; nothing else of epoch e-1 matters to it.  So a pair
// may start as soon as the two pairs of epoch e-1 that wrote its programs are
// done, while long-running pairs elsewhere are still being interpreted: the
// 8192-step tail of an epoch only delays its own dependency cone.
//
// Mechanics (one persistent launch for a run of epochs):
//  * work is claimed by warps in chunks of 32 consecutive pairs of one epoch,
//    in (epoch, pair) order, from one global counter;
//  * ver[p] counts the epochs of this run completed on program p; a lane
//    waits (acquire loads) until both its programs have ver == e, runs the
//    pair exactly as MutateAndRunPrograms does (common_language.h:163-192),
//    writes the tapes back and publishes ver = e + 1 with release stores;
//  * claims follow dependency order, so every chunk a warp waits on is
//    already held by a running warp: no deadlock;
//  * every wait is bounded (10 s of %globaltimer); a timeout sets *error, all
//    warps stop claiming, and the host reports CUBFF_ETIMEDOUT.
// Results are bit-identical to the per-epoch launches: every program sees the
// same sequence of pair operations with the same inputs.
#include <algorithm>

#include "epoch_body.cuh"

namespace cubff {
namespace {

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void fence_acq_rel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_volatile(const int *p) {
  return *reinterpret_cast<const volatile int *>(p);
}

constexpr uint64_t kWaitLimitNs = 10ull * 1000 * 1000 * 1000;

// Gather through L2 (ld.global.cg): the programs were written by other SMs
// during this launch.
__device__ __forceinline__ void load_pair_cg(const uint8_t *soup, uint32_t p1, uint32_t p2,
                                             uint32_t w[32]) {
  const uint4 *g1 = reinterpret_cast<const uint4 *>(soup + uint64_t(p1) * kTape);
  const uint4 *g2 = reinterpret_cast<const uint4 *>(soup + uint64_t(p2) * kTape);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const uint4 x = __ldcg(g1 + q);
    const uint4 y = __ldcg(g2 + q);
    w[4 * q + 0] = x.x; w[4 * q + 1] = x.y; w[4 * q + 2] = x.z; w[4 * q + 3] = x.w;
    w[16 + 4 * q + 0] = y.x; w[16 + 4 * q + 1] = y.y;
    w[16 + 4 * q + 2] = y.z; w[16 + 4 * q + 3] = y.w;
  }
}

// Mutation masks of MutateAndRunPrograms (common_language.h:172-180) for
// epochs [e0, e0 + E): bit i of mask[e][k] is set iff draw i of pair k,
// r = SplitMix64((n * seed(e0 + e) + k) * 128 + i), has bits [8, 38) below
// mutation_prob.  One thread per 32 draws; words are stored coalesced.
__global__ void mutation_mask_kernel(uint64_t s0, uint64_t e0, uint64_t npairs, uint64_t words,
                                     uint64_t n, uint32_t prob, uint32_t *out) {
  const uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= words) return;
  const uint64_t pair = idx >> 2, q = idx & 3;
  const uint64_t e = pair / npairs, k = pair - e * npairs;
  const uint64_t key0 = (n * seed_from(s0, e0 + e) + k) * kPair + q * 32;
  uint32_t m = 0;
#pragma unroll 8
  for (int b = 0; b < 32; b++) {
    const uint64_t r = splitmix64(key0 + b);
    m |= static_cast<uint32_t>((static_cast<uint32_t>(r >> 8) % (1u << 30)) < prob) << b;
  }
  out[idx] = m;
}

constexpr int kCountSlots = kPipeCountSlots;  // per-epoch counter slots (spread the atomics)
constexpr int kStepsPerVisit = 4;

// Lane-level dataflow.  Every lane runs pairs one after another; a pair
// depends only on the two pairs of the previous epoch that wrote its
// programs.  Tasks (epoch-major pair order) are dealt out in blocks of 32:
// warp w owns blocks w, w + W, w + 2W, ... (W = warps in the grid) and its
// lanes take the block's tasks in order as they become idle.  The lowest
// unfinished task is always runnable and either held by its owner warp or
// about to be taken by one of its idle lanes, so the pipeline cannot
// deadlock.
//
// No global access is consumed in the iteration that issues it: the next
// block's shuffle indices are loaded one block ahead, version polls are
// relaxed loads read back in the following iteration (with an acquire fence
// once a pair is ready), and a ready pair's gather lands in registers that
// are staged into shared memory in the following iteration.  Lane states:
// idle -> wait -> stage -> run -> (write back, publish) -> idle.
template <int L>
__global__ void __launch_bounds__(kThreads) lane_pipeline_kernel(PipeArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  constexpr bool kForthFam = LangTraits<L>::kForthFamily;
  constexpr bool kBffFam = (L <= kBffSelfmove);
  uint8_t *optab = smem + (kForthFam ? 2 : 1) * kGroups * kGroupBytes;
  uint8_t *cmdflag = optab + 256;
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  if (LangTraits<L>::kNeedsTable) {
    for (uint32_t c = tid; c < 256; c += kThreads) {
      optab[c] = op_of(L, c);
      cmdflag[c] = op_of(L, c) < kNull;
    }
  }
  __syncthreads();  // tables are read-only from here on; warps run independently
  const LaneBytes t{smem, lane_base(tid)};
  const LaneBytes stk{smem + kGroups * kGroupBytes, lane_base(tid)};
  const uint64_t npairs = a.n / 2;
  const uint64_t total = npairs * a.n_epochs;
  const uint64_t warp_id = uint64_t(blockIdx.x) * (kThreads / 32) + (tid >> 5);
  const uint64_t n_warps = uint64_t(gridDim.x) * (kThreads / 32);
  const uint32_t slot = static_cast<uint32_t>(warp_id % kCountSlots);
  const uint32_t lt_mask = (1u << lane) - 1;

  // Shuffle-index pair (p1 | p2 << 32) of task `task`, or 0 past the end.
  auto load_qp = [&](uint64_t task) -> uint64_t {
    if (task >= total) return 0;
    const uint64_t e = task / npairs, k = task - e * npairs;
    return *reinterpret_cast<const unsigned long long *>(a.perm + e * a.n + 2 * k);
  };
  uint64_t cur_block = warp_id, next_block = warp_id + n_warps;
  uint64_t cur_qp = load_qp(cur_block * 32 + lane);
  uint64_t next_qp = load_qp(next_block * 32 + lane);
  uint32_t used = 0;  // tasks of the current block already taken

  enum : uint32_t { kIdle = 0, kWait = 1, kStage = 2, kRun = 3, kDone = 4 };
  uint32_t state = kIdle, e = 0, p1 = 0, p2 = 0, v1 = 0, v2 = 0;
  uint64_t k = 0, t_wait = 0;
  uint32_t poll_gap = 1, poll_in = 0;  // per-lane poll backoff (iterations)
  uint32_t err = 0;                    // error flag as of the last poll
  bool dirty = false, evaluated = false;
  uint4 g[8];
  uint4 mm = make_uint4(0, 0, 0, 0);
  LaneMachine<L> m;

  while (true) {
    // 1. Idle lanes take the next tasks of the warp's blocks.
    const uint32_t idle = __ballot_sync(0xffffffffu, state == kIdle);
    if (idle) {
      const uint32_t idx = used + __popc(idle & lt_mask);
      const uint64_t qa = __shfl_sync(0xffffffffu, cur_qp, idx & 31);
      const uint64_t qb = __shfl_sync(0xffffffffu, next_qp, idx & 31);
      if (state == kIdle) {
        const uint64_t task = idx < 32 ? cur_block * 32 + idx : next_block * 32 + (idx - 32);
        if (task >= total) {
          state = kDone;
        } else {
          e = static_cast<uint32_t>(task / npairs);
          k = task - uint64_t(e) * npairs;
          const uint64_t qp = idx < 32 ? qa : qb;
          p1 = static_cast<uint32_t>(qp);
          p2 = static_cast<uint32_t>(qp >> 32);
          v1 = ld_relaxed(a.ver + p1);
          v2 = ld_relaxed(a.ver + p2);
          state = kWait;
          t_wait = 0;
          poll_gap = 1;
          poll_in = 0;
        }
      }
      used += __popc(idle);
      if (used >= 32) {  // current block exhausted: advance, prefetch the next
        used -= 32;
        cur_block = next_block;
        cur_qp = next_qp;
        next_block += n_warps;
        next_qp = load_qp(next_block * 32 + lane);
      }
    }
    if (__all_sync(0xffffffffu, state == kDone)) break;
    bool progressed = false;

    // 2. Staging: the gather issued in an earlier iteration has landed.
    if (state == kStage) {
      Mask128 cmd{0, 0};
#pragma unroll
      for (int q = 0; q < 32; q++) {
        const uint32_t w = q % 4 == 0 ? g[q / 4].x : q % 4 == 1 ? g[q / 4].y
                         : q % 4 == 2 ? g[q / 4].z : g[q / 4].w;
#pragma unroll
        for (int b = 0; b < 4; b++) t.set(4 * q + b, w >> (8 * b));
        if (kBffFam) {
          const uint32_t f = cmdflag[w & 0xFF] | (cmdflag[(w >> 8) & 0xFF] << 8) |
                             (cmdflag[(w >> 16) & 0xFF] << 16) | (cmdflag[w >> 24] << 24);
          const uint64_t nib = (f * 0x01020408u) >> 24;
          if (q < 16) cmd.lo |= nib << (4 * q);
          else cmd.hi |= nib << (4 * (q - 16));
        }
      }
      dirty = (mm.x | mm.y | mm.z | mm.w) != 0;
      if (dirty) {
        const uint64_t key0 = (a.n * seed_from(a.s0, a.e0 + e) + k) * kPair;
        const uint32_t mw[4] = {mm.x, mm.y, mm.z, mm.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
          uint32_t bits = mw[q];
          while (bits) {
            const int i = q * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
            const uint32_t v = static_cast<uint32_t>(splitmix64(key0 + i)) & 0xFFu;
            t.set(i, v);
            if (kBffFam) mask_assign(cmd, i, cmdflag[v] != 0);
          }
        }
      }
      const uint64_t num_indices = a.d_num_indices ? a.d_num_indices[e] : npairs;
      evaluated = k < num_indices;
      m.begin(t, cmd);
      state = kRun;
      progressed = true;
    } else if (state == kWait) {
      // 3. Waiting: versions polled in the previous iteration.
      if (v1 >= e && v2 >= e) {
        fence_acq_rel_gpu();  // order the gather after the observed releases
        const uint4 *g1 = reinterpret_cast<const uint4 *>(a.soup + uint64_t(p1) * kTape);
        const uint4 *g2 = reinterpret_cast<const uint4 *>(a.soup + uint64_t(p2) * kTape);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          g[q] = __ldcg(g1 + q);
          g[4 + q] = __ldcg(g2 + q);
        }
        mm = __ldg(a.mutmask + uint64_t(e) * npairs + k);
        state = kStage;
        progressed = true;
      } else if (poll_in-- == 0) {
        // Not ready: the error flag and the deadline are checked on the poll
        // schedule, and the next poll is issued (read back next time).
        if (err) {
          state = kDone;
        } else {
          const uint64_t now = globaltimer_ns();
          if (t_wait == 0) {
            t_wait = now;
          } else if (now - t_wait > kWaitLimitNs) {
            atomicExch(a.error, 1);
            state = kDone;
          }
        }
        if (state == kWait) {
          v1 = ld_relaxed(a.ver + p1);
          v2 = ld_relaxed(a.ver + p2);
          err = ld_relaxed(reinterpret_cast<const uint32_t *>(a.error));
          poll_gap = poll_gap < 16 ? poll_gap * 2 : 16;
          poll_in = poll_gap;
        }
      }
    } else if (state == kRun) {
      // 4. Running: a few interpreter steps; finish with write-back + publish.
      progressed = true;
      bool fin = !evaluated;
      for (int r = 0; r < kStepsPerVisit && !fin; r++) fin = m.step(t, stk, optab);
      if (fin) {
        if (dirty || (evaluated && m.mods() != 0)) {
          uint32_t w[32];
#pragma unroll
          for (int q = 0; q < 32; q++)
            w[q] = t.get(4 * q) | (t.get(4 * q + 1) << 8) | (t.get(4 * q + 2) << 16) |
                   (t.get(4 * q + 3) << 24);
          // First half, then second half (common_language.h:188-191).
          uint4 *o1 = reinterpret_cast<uint4 *>(a.soup + uint64_t(p1) * kTape);
          uint4 *o2 = reinterpret_cast<uint4 *>(a.soup + uint64_t(p2) * kTape);
#pragma unroll
          for (int q = 0; q < 4; q++)
            o1[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
#pragma unroll
          for (int q = 0; q < 4; q++)
            o2[q] = make_uint4(w[16 + 4 * q], w[16 + 4 * q + 1], w[16 + 4 * q + 2],
                               w[16 + 4 * q + 3]);
        }
        st_release(a.ver + p1, e + 1);  // orders the tape stores before the flags
        st_release(a.ver + p2, e + 1);
        if (evaluated) {
          unsigned long long *c = a.ops + (uint64_t(e) * kCountSlots + slot) * 2;
          if (m.ops()) atomicAdd(c, static_cast<unsigned long long>(m.ops()));
          if (m.raw()) atomicAdd(c + 1, static_cast<unsigned long long>(m.raw()));
        }
        state = kIdle;
      }
    }
    if (!__any_sync(0xffffffffu, progressed)) __nanosleep(200);
  }
}

}  // namespace

int launch_mutation_masks(uint64_t s0, uint64_t e0, uint32_t n_epochs, uint64_t n, uint32_t prob,
                          uint4 *out, cudaStream_t stream) {
  const uint64_t words = (n / 2) * n_epochs * 4;
  if (words == 0) return CUBFF_OK;
  mutation_mask_kernel<<<static_cast<unsigned>((words + 255) / 256), 256, 0, stream>>>(
      s0, e0, n / 2, words, n, prob, reinterpret_cast<uint32_t *>(out));
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

namespace {
template <int L>
int launch_pipeline_t(const PipeArgs &a, int device, cudaStream_t stream) {
  static int grid_cache[64] = {0};
  int &g = grid_cache[device & 63];
  const size_t smem = epoch_smem_bytes<L>() + 256;
  if (g == 0) {
    int per_sm = 0, sms = 0;
    CUBFF_CUDA_TRY(cudaFuncSetAttribute(lane_pipeline_kernel<L>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem)));
    CUBFF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lane_pipeline_kernel<L>,
                                                                 kThreads, smem));
    CUBFF_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    g = std::max(1, per_sm) * sms;
  }
  // Lanes in flight: enough to keep the SMs busy, few enough that most held
  // pairs are ready (a lane holding a pair of a later epoch only polls).
  // lanes_per_pair (x1/64) is tunable; the default keeps half an epoch of
  // pairs in flight.
  const uint64_t npairs = a.n / 2;
  uint64_t want = (npairs * static_cast<uint64_t>(a.lanes_per_pair64 ? a.lanes_per_pair64 : 32)) / 64;
  want = std::max<uint64_t>(want, kThreads);
  const uint64_t blocks = (want + kThreads - 1) / kThreads;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(blocks, uint64_t(g)));
  lane_pipeline_kernel<L><<<grid, kThreads, smem, stream>>>(a);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

template <int L>
struct PipeLauncher {
  static int run(const PipeArgs &a, int device, cudaStream_t s) {
    return launch_pipeline_t<L>(a, device, s);
  }
};

}  // namespace

int launch_pipeline(int lang, const PipeArgs &a, int device, cudaStream_t stream) {
  if (a.n < 2 || a.n_epochs == 0) return CUBFF_OK;

  switch (lang) {
    case kBff: return PipeLauncher<kBff>::run(a, device, stream);
    case kBffNoheads: return PipeLauncher<kBffNoheads>::run(a, device, stream);
    case kBffNoheads4bit: return PipeLauncher<kBffNoheads4bit>::run(a, device, stream);
    case kBffPerm: return PipeLauncher<kBffPerm>::run(a, device, stream);
    case kBff8: return PipeLauncher<kBff8>::run(a, device, stream);
    case kBff8Noheads: return PipeLauncher<kBff8Noheads>::run(a, device, stream);
    case kBffSelfmove: return PipeLauncher<kBffSelfmove>::run(a, device, stream);
    case kForth: return PipeLauncher<kForth>::run(a, device, stream);
    case kForthcopy: return PipeLauncher<kForthcopy>::run(a, device, stream);
    case kForthtrivial: return PipeLauncher<kForthtrivial>::run(a, device, stream);
    case kForthtrivialReset: return PipeLauncher<kForthtrivialReset>::run(a, device, stream);
    case kSubleq: return PipeLauncher<kSubleq>::run(a, device, stream);
    case kRsubleq4: return PipeLauncher<kRsubleq4>::run(a, device, stream);
  }
  return set_error(CUBFF_ENOTFOUND, "unknown language id %d", lang);
}

}  // namespace cubff
