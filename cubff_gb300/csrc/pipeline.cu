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
constexpr int kStepsPerVisit = 8;
constexpr int kStepsLong = 64;
constexpr uint32_t kLongRaw = 256;

// Ready-queue dataflow.  A pair of epoch e+1 can run once the two pairs of
// epoch e that wrote its programs are done.  A finished pair notifies the
// consumers of its two programs (inv gives a program's position in the next
// epoch's shuffle, hence its pair); the second notification of a consumer
// pushes it into the ready queue.  Warps claim queue slots in bulk, so the
// lanes they hand out stage their pairs together; epoch-0 pairs of the run
// are implicitly ready (slots [0, npairs)).  Every pushed task is runnable,
// so no lane ever waits on a dependency; a lane only waits for a claimed
// slot to be filled, and every slot below the task count is eventually
// filled (all pairs of epoch e complete => all of epoch e+1 are pushed).
//
// No global access is consumed in the iteration that issues it where that
// can be avoided: queue entries, shuffle indices and gathers land in
// registers read back in a later iteration.  Lane states:
//   idle -> slot (wait for the entry) -> index -> stage -> run -> notify -> idle.
constexpr int kClaimMin = 8;

__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t *p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int L>
__global__ void __launch_bounds__(kThreads) lane_pipeline_kernel(PipeArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  constexpr bool kBffFam = (L <= kBffSelfmove);
  uint8_t *optab = smem + 2 * kGroups * kGroupBytes;
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
  const uint32_t npairs = static_cast<uint32_t>(a.n / 2);
  const uint32_t n_ep = a.n_epochs;
  const uint32_t total = npairs * n_ep;
  const uint64_t warp_id = uint64_t(blockIdx.x) * (kThreads / 32) + (tid >> 5);
  const uint32_t slot_ctr = static_cast<uint32_t>(warp_id % kCountSlots);
  const uint32_t lt_mask = (1u << lane) - 1;

  enum : uint32_t { kIdle, kSlot, kIndex, kStage, kRun, kNotify, kDone };
  uint32_t state = kIdle, slot = 0, task = 0, e = 0, k = 0, p1 = 0, p2 = 0;
  uint32_t qv = 0, poll_gap = 1, poll_in = 0, err = 0;
  uint32_t j1 = 0, j2 = 0, c1 = 0, c2 = 0;
  uint64_t qp = 0, t_wait = 0;
  bool dirty = false, evaluated = false;
  uint4 g[8];
  uint4 mm = make_uint4(0, 0, 0, 0);
  LaneMachine<L> m;

  while (true) {
    // 1. Bulk claim of queue slots by idle lanes.
    const uint32_t idle = __ballot_sync(0xffffffffu, state == kIdle);
    const uint32_t busy = __ballot_sync(0xffffffffu, state != kIdle && state != kDone);
    if (idle && (__popc(idle) >= kClaimMin || busy == 0)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == static_cast<uint32_t>(leader)) base = atomicAdd(a.qctl, __popc(idle));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (state == kIdle) {
        slot = base + __popc(idle & lt_mask);
        if (slot >= total) {
          state = kDone;
        } else if (slot < npairs) {  // an epoch-0 pair of the run: ready
          task = slot;
          state = kIndex;
          qp = *reinterpret_cast<const unsigned long long *>(a.perm + 2 * uint64_t(task));
        } else {
          state = kSlot;
          qv = ld_relaxed(a.queue + (slot - npairs));
          poll_gap = 1;
          poll_in = 0;
          t_wait = 0;
        }
      }
    }
    if (__all_sync(0xffffffffu, state == kDone)) break;
    bool progressed = false;

    if (state == kSlot) {
      // 2. Waiting for the claimed slot's entry (polled in an earlier iteration).
      if (qv != 0) {
        task = qv - 1;
        e = task / npairs;
        qp = *reinterpret_cast<const unsigned long long *>(
            a.perm + uint64_t(e) * a.n + 2 * uint64_t(task - e * npairs));
        state = kIndex;
        progressed = true;
      } else if (poll_in-- == 0) {
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
        if (state == kSlot) {
          qv = ld_relaxed(a.queue + (slot - npairs));
          err = ld_relaxed(reinterpret_cast<const uint32_t *>(a.error));
          poll_gap = poll_gap < 16 ? poll_gap * 2 : 16;
          poll_in = poll_gap;
        }
      }
    } else if (state == kIndex) {
      // 3. Shuffle indices landed: order after the producers, issue the gather,
      //    the mutation mask and the next epoch's positions of both programs.
      e = task / npairs;
      k = task - e * npairs;
      p1 = static_cast<uint32_t>(qp);
      p2 = static_cast<uint32_t>(qp >> 32);
      fence_acq_rel_gpu();
      const uint4 *g1 = reinterpret_cast<const uint4 *>(a.soup + uint64_t(p1) * kTape);
      const uint4 *g2 = reinterpret_cast<const uint4 *>(a.soup + uint64_t(p2) * kTape);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        g[q] = __ldcg(g1 + q);
        g[4 + q] = __ldcg(g2 + q);
      }
      mm = __ldg(a.mutmask + task);
      if (e + 1 < n_ep) {
        j1 = __ldg(a.inv + uint64_t(e + 1) * a.n + p1);
        j2 = __ldg(a.inv + uint64_t(e + 1) * a.n + p2);
      }
      state = kStage;
      progressed = true;
    } else if (state == kStage) {
      // 4. Stage the pair: bytes into shared memory, command mask, mutations.
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
    } else if (state == kRun) {
      // 5. A few interpreter steps; on the end, write back and notify.
      progressed = true;
      bool fin = !evaluated;
      // Pairs that have run long are the ones later epochs wait on: give
      // them more steps per visit of the warp.
      const int steps = m.raw() > kLongRaw ? kStepsLong : kStepsPerVisit;
      for (int r = 0; r < steps && !fin; r++) fin = m.step(t, stk, optab);
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
        if (evaluated) {
          unsigned long long *c = a.ops + (uint64_t(e) * kCountSlots + slot_ctr) * 2;
          if (m.ops()) atomicAdd(c, static_cast<unsigned long long>(m.ops()));
          if (m.raw()) atomicAdd(c + 1, static_cast<unsigned long long>(m.raw()));
        }
        if (e + 1 < n_ep) {
          // The acq_rel increments order the stores above before them, and
          // make the earlier producer's stores visible to whoever pushes.
          uint32_t *rc = a.readycnt + uint64_t(e + 1) * npairs;
          c1 = atom_add_acq_rel(rc + (j1 >> 1), 1);
          c2 = atom_add_acq_rel(rc + (j2 >> 1), 1);
          state = kNotify;
        } else {
          state = kIdle;
        }
      }
    }
    // 6. Push the consumers whose second input this pair was.
    const bool push1 = state == kNotify && c1 == 1;
    const bool push2 = state == kNotify && c2 == 1 && (j2 >> 1) != (j1 >> 1);
    const bool push1b = state == kNotify && c2 == 1 && (j2 >> 1) == (j1 >> 1);
    const uint32_t nmask1 = __ballot_sync(0xffffffffu, push1 || push1b);
    const uint32_t nmask2 = __ballot_sync(0xffffffffu, push2);
    if (nmask1 | nmask2) {
      const int leader = __ffs(nmask1 | nmask2) - 1;
      uint32_t base = 0;
      if (lane == static_cast<uint32_t>(leader))
        base = atomicAdd(a.qctl + 1, __popc(nmask1) + __popc(nmask2));
      base = __shfl_sync(0xffffffffu, base, leader);
      const uint32_t next = (e + 1) * npairs;
      if (push1 || push1b)
        st_release_u32(a.queue + base + __popc(nmask1 & lt_mask), next + (j1 >> 1) + 1);
      if (push2)
        st_release_u32(a.queue + base + __popc(nmask1) + __popc(nmask2 & lt_mask),
                       next + (j2 >> 1) + 1);
    }
    if (state == kNotify) state = kIdle;
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

// ---------------------------------------------------------------------------
// Kernel-level pipelined run on caller-owned buffers (cubff_run_epochs).

namespace cubff {
namespace {

struct RunWs {
  uint4 *mutmask;
  uint32_t *inv, *readycnt, *queue, *ctl;
  unsigned long long *counters;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

RunWs run_ws(void *base, uint64_t n, uint32_t E) {
  const uint64_t P = n / 2;
  uint8_t *p = static_cast<uint8_t *>(base);
  RunWs w;
  w.mutmask = reinterpret_cast<uint4 *>(p);
  p += align256(size_t(E) * P * sizeof(uint4));
  w.inv = reinterpret_cast<uint32_t *>(p);
  p += align256(size_t(E) * n * sizeof(uint32_t));
  w.readycnt = reinterpret_cast<uint32_t *>(p);
  p += align256(size_t(E) * P * sizeof(uint32_t));
  w.queue = reinterpret_cast<uint32_t *>(p);
  p += align256(size_t(E) * P * sizeof(uint32_t));
  w.counters = reinterpret_cast<unsigned long long *>(p);
  p += align256(size_t(E) * kPipeCountSlots * 2 * sizeof(unsigned long long));
  w.ctl = reinterpret_cast<uint32_t *>(p);
  return w;
}

// d_counts[e] += the per-slot counters of epoch e.
__global__ void reduce_counts_kernel(const unsigned long long *slots, uint32_t E,
                                     unsigned long long *out) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  unsigned long long o = 0, r = 0;
  for (int s = 0; s < kPipeCountSlots; s++) {
    o += slots[(uint64_t(e) * kPipeCountSlots + s) * 2];
    r += slots[(uint64_t(e) * kPipeCountSlots + s) * 2 + 1];
  }
  out[2 * e] += o;
  out[2 * e + 1] += r;
}

}  // namespace
}  // namespace cubff

extern "C" size_t cubff_run_epochs_workspace_bytes(uint64_t num_programs, uint32_t n_epochs) {
  using namespace cubff;
  const uint64_t P = num_programs / 2;
  return align256(size_t(n_epochs) * P * sizeof(uint4)) +
         align256(size_t(n_epochs) * num_programs * sizeof(uint32_t)) +
         2 * align256(size_t(n_epochs) * P * sizeof(uint32_t)) +
         align256(size_t(n_epochs) * kPipeCountSlots * 2 * sizeof(unsigned long long)) + 256;
}

extern "C" int cubff_run_epochs(int lang, uint8_t *d_programs, const uint32_t *d_shuf_idx,
                                const uint64_t *d_num_indices, uint64_t params_seed,
                                uint64_t first_epoch, uint32_t n_epochs, uint32_t mutation_prob,
                                uint64_t num_programs, unsigned long long *d_counts,
                                void *d_workspace, size_t workspace_bytes, void *stream) {
  using namespace cubff;
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  if (!d_programs || !d_shuf_idx || !d_counts || !d_workspace || num_programs < 2 ||
      num_programs % 2 != 0 || num_programs > (1ull << 31))
    return set_error(CUBFF_EINVAL, "run_epochs: bad arguments");
  if ((reinterpret_cast<uintptr_t>(d_programs) & 15) || (reinterpret_cast<uintptr_t>(d_shuf_idx) & 7) ||
      (reinterpret_cast<uintptr_t>(d_workspace) & 255))
    return set_error(CUBFF_EINVAL, "run_epochs: misaligned buffer (programs 16, indices 8, "
                                   "workspace 256 bytes)");
  if (workspace_bytes < cubff_run_epochs_workspace_bytes(num_programs, n_epochs))
    return set_error(CUBFF_EINVAL, "run_epochs: workspace too small (%zu < %zu)", workspace_bytes,
                     cubff_run_epochs_workspace_bytes(num_programs, n_epochs));
  if (n_epochs == 0) return CUBFF_OK;
  if ((num_programs / 2) * uint64_t(n_epochs) >= (1ull << 32))
    return set_error(CUBFF_EINVAL, "run_epochs: num_programs/2 * n_epochs must be < 2^32");
  int dev = 0;
  CUBFF_CUDA_TRY(cudaGetDevice(&dev));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t n = num_programs, P = n / 2, s0 = splitmix64(params_seed);
  RunWs w = run_ws(d_workspace, n, n_epochs);
  CUBFF_CUDA_TRY(cudaMemsetAsync(w.readycnt, 0, size_t(n_epochs) * P * sizeof(uint32_t), st));
  CUBFF_CUDA_TRY(cudaMemsetAsync(w.queue, 0, size_t(n_epochs) * P * sizeof(uint32_t), st));
  CUBFF_CUDA_TRY(cudaMemsetAsync(w.counters, 0,
                                 size_t(n_epochs) * kPipeCountSlots * 2 * sizeof(unsigned long long), st));
  CUBFF_CUDA_TRY(cudaMemsetAsync(w.ctl, 0, 4 * sizeof(uint32_t), st));
  CUBFF_TRY(launch_mutation_masks(s0, first_epoch, n_epochs, n, mutation_prob, w.mutmask, st));
  CUBFF_TRY(launch_inverse(d_shuf_idx, n_epochs, n, w.inv, st));
  PipeArgs a;
  a.soup = d_programs;
  a.perm = d_shuf_idx;
  a.n = n;
  a.s0 = s0;
  a.e0 = first_epoch;
  a.n_epochs = n_epochs;
  a.mutation_prob = mutation_prob;
  a.d_num_indices = d_num_indices;
  a.mutmask = w.mutmask;
  a.inv = w.inv;
  a.readycnt = w.readycnt;
  a.queue = w.queue;
  a.qctl = w.ctl;
  a.error = reinterpret_cast<int *>(w.ctl + 2);
  a.ops = w.counters;
  a.lanes_per_pair64 = 0;
  CUBFF_TRY(launch_pipeline(lang, a, dev, st));
  reduce_counts_kernel<<<(n_epochs + 127) / 128, 128, 0, st>>>(w.counters, n_epochs, d_counts);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

extern "C" int cubff_run_epochs_status(const void *d_workspace, uint64_t num_programs,
                                       uint32_t n_epochs, void *stream) {
  using namespace cubff;
  if (!d_workspace) return set_error(CUBFF_EINVAL, "run_epochs_status: null workspace");
  RunWs w = run_ws(const_cast<void *>(d_workspace), num_programs, n_epochs);
  int err = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CUBFF_CUDA_TRY(cudaMemcpyAsync(&err, w.ctl + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(st));
  if (err) return set_error(CUBFF_ETIMEDOUT, "run_epochs: a pipelined wait timed out");
  return CUBFF_OK;
}
