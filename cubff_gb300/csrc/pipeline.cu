// pipeline.cu — epochs of one or more soups run as one dataflow pipeline
// instead of one launch per epoch.
//
// Pair k of epoch e reads programs s_e[2k], s_e[2k+1] as epoch e-1 left them
// and writes them back; nothing else of epoch e-1 matters to it.  So a pair
// may start as soon as the two pairs of epoch e-1 that wrote its programs are
// done, while long-running pairs elsewhere are still being interpreted: the
// 8192-step tail of an epoch only delays its own dependency cone.  Soups are
// independent, so a batch of soups of one language (any sizes and mutation
// rates) shares one persistent launch and one ready queue.
//
// Every wait is bounded (10 s of %globaltimer by default); a timeout sets
// *error = 1, the waiting lanes give up, and the host reports CUBFF_ETIMEDOUT.
// A ready-queue entry naming no task of the launch sets *error = 2 (reported
// as CUBFF_EDEVICE) instead of being used as an index.  Results are
// bit-identical to the per-epoch launches: every program sees the same
// sequence of pair operations (MutateAndRunPrograms, common_language.h:163-192)
// with the same inputs.
#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "epoch_body.cuh"

namespace cubff {
namespace {

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void fence_acq_rel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr uint64_t kDefaultWaitLimitNs = 10ull * 1000 * 1000 * 1000;
std::atomic<uint64_t> g_wait_limit_ns{kDefaultWaitLimitNs};

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

// Ready-queue dataflow over one or more soups.  A pair of epoch e+1 can run
// once the two pairs of epoch e that wrote its programs are done.  A finished
// pair notifies the consumers of its two programs (inv gives a program's
// position in the next epoch's shuffle, hence its pair); the second
// notification of a consumer pushes it into its language's ready queue.
// Epoch-0 pairs of the launch are implicitly ready (the first `initial`
// slots of each queue).  Warps claim queue slots in bulk, so the lanes they
// hand out stage their pairs together.  Every pushed task is runnable, so no
// lane ever waits on a dependency; a lane only waits for a claimed slot to be
// written, and every slot below a queue's task count is eventually written
// (all pairs of epoch e complete => all of epoch e+1 are pushed).
//
// A launch serves the soups of one language through one queue (the soups of
// other languages run in launches of their own, on other streams).
//
// No global access is consumed in the iteration that issues it where that
// can be avoided: queue entries, shuffle indices and gathers land in
// registers read back in a later iteration.  Lane states:
//   idle -> slot (wait for the entry) -> index -> stage -> run -> notify -> idle
// and `exhausted` once a claim falls past the queue's last task.
//
// Launch-shape knobs (PipeTuning, chosen by the host):
//  * steps_per_visit: interpreter steps a running lane takes per iteration of
//    its warp after its first (an iteration lasts as long as its busiest
//    lane, so a lane given more steps holds its warp-mates, and the pairs
//    they would finish and notify, for its extra steps);
//  * first_visit_steps: the steps of a pair's first visit.  Lanes that claim
//    together stage and start together, and most pairs end within a few
//    steps; the first visit's budget bounds how long one heavy pair among
//    them holds the others (whose consumers wait on them) before they can
//    write back;
//  * claim_min: a warp with running lanes claims new slots only once this
//    many of its lanes are idle (an idle warp claims at once), so a slot held
//    by a busy warp is polled only between its long iterations;
//  * long_visits: a pair still running after this many visits is long.  A
//    warp holding a long pair claims nothing new: its other lanes drain, and
//    the long pair, which the next epochs' pairs wait on, steps without
//    warp-mates whose staging and steps would interleave with its own.  Few
//    pairs are long (a random 2^17-program soup has ~10-25 pairs per epoch
//    past 64 steps, out of 65536), so little capacity is set aside.

__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t *p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

enum : uint32_t { kIdle, kSlot, kIndex, kStage, kRun, kNotify, kExhausted };

// Per-lane state that does not depend on the language.
struct Lane {
  uint32_t state, slot, task, e, k, p1, p2, qv, poll_gap, poll_in, err, j1, j2, c1, c2, visits;
  int si;  // soup index of the task
  uint64_t qp, t_wait;
  bool dirty, evaluated, has_next;
  uint4 g[8];
  uint4 mm;
};

// What a warp needs of the launch: the soup descriptors (in shared memory)
// and the error flag.
struct PipeCtx {
  const PipeSoup *soups;
  int *error;
  uint64_t wait_limit_ns;
  PipeTuning tune;
};

// Soup of global task `task` among soups [lo, hi) (sorted by task_base).
__device__ __forceinline__ int soup_of_task(const PipeSoup *soups, int lo, int hi, uint32_t task) {
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (soups[mid].task_base <= task) lo = mid; else hi = mid;
  }
  return lo;
}

// Soup of epoch-0 slot `slot` among soups [lo, hi) (sorted by init_base).
__device__ __forceinline__ int soup_of_slot(const PipeSoup *soups, int lo, int hi, uint32_t slot) {
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (soups[mid].init_base <= slot) lo = mid; else hi = mid;
  }
  return lo;
}

// One iteration of a warp serving language L.  Returns true if a lane made
// progress.
template <int L>
__device__ __forceinline__ bool iterate(const PipeCtx &b, const PipeQueue &q, Lane &ln,
                                        LaneMachine<L> &m, const LaneBytes t, const LaneBytes stk,
                                        const LaneNp np, const uint8_t *__restrict__ optab,
                                        const uint8_t *__restrict__ cmdflag, uint32_t lane,
                                        uint32_t slot_ctr) {
  constexpr bool kBffFam = (L <= kBffSelfmove);
  const uint32_t lt_mask = (1u << lane) - 1;
  const int s_lo = static_cast<int>(q.first_soup), s_hi = static_cast<int>(q.first_soup + q.n_soups);

  // 1. Bulk claim of queue slots by idle lanes.
  const uint32_t idle = __ballot_sync(0xffffffffu, ln.state == kIdle);
  const uint32_t busy = __ballot_sync(0xffffffffu, ln.state != kIdle && ln.state != kExhausted);
  const uint32_t lng = __ballot_sync(0xffffffffu, ln.state == kRun && ln.visits >= b.tune.long_visits);
  if (idle && (busy == 0 || (lng == 0 && __popc(idle) >= b.tune.claim_min))) {
    const int leader = __ffs(idle) - 1;
    uint32_t base = 0;
    if (lane == static_cast<uint32_t>(leader)) base = atomicAdd(q.ctl, __popc(idle));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (ln.state == kIdle) {
      ln.slot = base + __popc(idle & lt_mask);
      if (ln.slot >= q.total) {
        ln.state = kExhausted;
      } else if (ln.slot < q.initial) {  // a first-epoch pair: ready
        ln.si = soup_of_slot(b.soups, s_lo, s_hi, ln.slot);
        const PipeSoup &sp = b.soups[ln.si];
        ln.task = sp.task_base + (ln.slot - sp.init_base);
        ln.state = kIndex;
        ln.qp = *reinterpret_cast<const unsigned long long *>(sp.perm + 2 * uint64_t(ln.slot - sp.init_base));
      } else {
        ln.state = kSlot;
        ln.qv = ld_relaxed(q.queue + (ln.slot - q.initial));
        ln.poll_gap = 1;
        ln.poll_in = 0;
        ln.t_wait = 0;
      }
    }
  }
  bool progressed = false;

  if (ln.state == kSlot) {
    // 2. Waiting for the claimed slot's entry (polled in an earlier iteration).
    if (ln.qv != 0 && ln.qv - 1 >= q.total) {
      // Only pushes of tasks of this launch fill the queue; any other value
      // is reported (error 2) instead of being used as an index.
      atomicExch(b.error, 2);
      ln.state = kExhausted;
    } else if (ln.qv != 0) {
      ln.task = ln.qv - 1;
      // Consumed: leave the entry zero for the next launch.
      q.queue[ln.slot - q.initial] = 0;
      ln.si = soup_of_task(b.soups, s_lo, s_hi, ln.task);
      const PipeSoup &sp = b.soups[ln.si];
      const uint32_t rel = ln.task - sp.task_base;
      ln.e = rel / sp.npairs;
      ln.k = rel - ln.e * sp.npairs;
      ln.qp = *reinterpret_cast<const unsigned long long *>(sp.perm + uint64_t(ln.e) * sp.n +
                                                            2 * uint64_t(ln.k));
      ln.state = kIndex;
      progressed = true;
    } else if (ln.poll_in-- == 0) {
      if (ln.err) {
        ln.state = kExhausted;
      } else {
        const uint64_t now = globaltimer_ns();
        if (ln.t_wait == 0) {
          ln.t_wait = now;
        } else if (now - ln.t_wait > b.wait_limit_ns) {
          atomicExch(b.error, 1);
          ln.state = kExhausted;
        }
      }
      if (ln.state == kSlot) {
        ln.qv = ld_relaxed(q.queue + (ln.slot - q.initial));
        ln.err = ld_relaxed(reinterpret_cast<const uint32_t *>(b.error));
        ln.poll_gap = ln.poll_gap < 16 ? ln.poll_gap * 2 : 16;
        ln.poll_in = ln.poll_gap;
      }
    }
  } else if (ln.state == kIndex) {
    // 3. Shuffle indices landed: order after the producers, issue the gather,
    //    the mutation mask and the next epoch's positions of both programs.
    const PipeSoup &sp = b.soups[ln.si];
    if (ln.slot < q.initial) {
      ln.e = 0;
      ln.k = ln.slot - sp.init_base;
    }
    ln.p1 = static_cast<uint32_t>(ln.qp);
    ln.p2 = static_cast<uint32_t>(ln.qp >> 32);
    fence_acq_rel_gpu();
    // Both inputs have been counted: leave the counter zero for the next launch.
    if (ln.e > 0) sp.readycnt[uint64_t(ln.e) * sp.npairs + ln.k] = 0;
    const uint4 *g1 = reinterpret_cast<const uint4 *>(sp.soup + uint64_t(ln.p1) * kTape);
    const uint4 *g2 = reinterpret_cast<const uint4 *>(sp.soup + uint64_t(ln.p2) * kTape);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      ln.g[i] = __ldcg(g1 + i);
      ln.g[4 + i] = __ldcg(g2 + i);
    }
    ln.mm = __ldg(sp.mutmask + uint64_t(ln.e) * sp.npairs + ln.k);
    ln.has_next = ln.e + 1 < sp.n_epochs;
    if (ln.has_next) {
      ln.j1 = __ldg(sp.inv + uint64_t(ln.e + 1) * sp.n + ln.p1);
      ln.j2 = __ldg(sp.inv + uint64_t(ln.e + 1) * sp.n + ln.p2);
    }
    ln.state = kStage;
    progressed = true;
  } else if (ln.state == kStage) {
    // 4. Stage the pair: bytes into shared memory, command mask, mutations.
    const PipeSoup &sp = b.soups[ln.si];
    Mask128 cmd{0, 0};
#pragma unroll
    for (int qd = 0; qd < 32; qd++) {
      const uint32_t w = qd % 4 == 0 ? ln.g[qd / 4].x : qd % 4 == 1 ? ln.g[qd / 4].y
                       : qd % 4 == 2 ? ln.g[qd / 4].z : ln.g[qd / 4].w;
#pragma unroll
      for (int bb = 0; bb < 4; bb++) t.set(4 * qd + bb, w >> (8 * bb));
      if (kBffFam) {
        const uint32_t f = cmdflag[w & 0xFF] | (cmdflag[(w >> 8) & 0xFF] << 8) |
                           (cmdflag[(w >> 16) & 0xFF] << 16) | (cmdflag[w >> 24] << 24);
        const uint64_t nib = (f * 0x01020408u) >> 24;
        if (qd < 16) cmd.lo |= nib << (4 * qd);
        else cmd.hi |= nib << (4 * (qd - 16));
      }
    }
    ln.dirty = (ln.mm.x | ln.mm.y | ln.mm.z | ln.mm.w) != 0;
    if (ln.dirty) {
      const uint64_t key0 = (sp.n * seed_from(sp.s0, sp.e0 + ln.e) + ln.k) * kPair;
      const uint32_t mw[4] = {ln.mm.x, ln.mm.y, ln.mm.z, ln.mm.w};
#pragma unroll
      for (int qd = 0; qd < 4; qd++) {
        uint32_t bits = mw[qd];
        while (bits) {
          const int i = qd * 32 + __ffs(bits) - 1;
          bits &= bits - 1;
          const uint32_t v = static_cast<uint32_t>(splitmix64(key0 + i)) & 0xFFu;
          t.set(i, v);
          if (kBffFam) mask_assign(cmd, i, cmdflag[v] != 0);
        }
      }
    }
    const uint64_t num_indices = sp.num_indices ? sp.num_indices[ln.e] : sp.npairs;
    ln.evaluated = ln.k < num_indices;
    m.begin(t, cmd);
    ln.visits = 0;
    ln.state = kRun;
    progressed = true;
  } else if (ln.state == kRun) {
    // 5. A few interpreter steps; on the end, write back and notify.
    progressed = true;
    bool fin = !ln.evaluated;
    const uint32_t steps = ln.visits ? b.tune.steps_per_visit : b.tune.first_visit_steps;
    for (uint32_t r = 0; r < steps && !fin; r++) fin = m.step(t, stk, np, optab);
    ln.visits++;
    if (fin) {
      const PipeSoup &sp = b.soups[ln.si];
      if (ln.dirty || (ln.evaluated && m.mods() != 0)) {
        uint32_t w[32];
#pragma unroll
        for (int qd = 0; qd < 32; qd++)
          w[qd] = t.get(4 * qd) | (t.get(4 * qd + 1) << 8) | (t.get(4 * qd + 2) << 16) |
                  (t.get(4 * qd + 3) << 24);
        // First half, then second half (common_language.h:188-191).
        uint4 *o1 = reinterpret_cast<uint4 *>(sp.soup + uint64_t(ln.p1) * kTape);
        uint4 *o2 = reinterpret_cast<uint4 *>(sp.soup + uint64_t(ln.p2) * kTape);
#pragma unroll
        for (int qd = 0; qd < 4; qd++)
          o1[qd] = make_uint4(w[4 * qd], w[4 * qd + 1], w[4 * qd + 2], w[4 * qd + 3]);
#pragma unroll
        for (int qd = 0; qd < 4; qd++)
          o2[qd] = make_uint4(w[16 + 4 * qd], w[16 + 4 * qd + 1], w[16 + 4 * qd + 2],
                              w[16 + 4 * qd + 3]);
      }
      if (ln.evaluated) {
        unsigned long long *c = sp.ops + (uint64_t(ln.e) * kCountSlots + slot_ctr) * 2;
        if (m.ops()) atomicAdd(c, static_cast<unsigned long long>(m.ops()));
        if (m.raw()) atomicAdd(c + 1, static_cast<unsigned long long>(m.raw()));
      }
      if (ln.has_next) {
        // The acq_rel increments order the stores above before them, and make
        // the earlier producer's stores visible to whoever pushes.
        uint32_t *rc = sp.readycnt + uint64_t(ln.e + 1) * sp.npairs;
        ln.c1 = atom_add_acq_rel(rc + (ln.j1 >> 1), 1);
        ln.c2 = atom_add_acq_rel(rc + (ln.j2 >> 1), 1);
        ln.state = kNotify;
      } else {
        ln.state = kIdle;
      }
    }
  }
  // 6. Push the consumers whose second input this pair was.
  const bool same = (ln.j2 >> 1) == (ln.j1 >> 1);
  const bool push1 = ln.state == kNotify && (ln.c1 == 1 || (same && ln.c2 == 1));
  const bool push2 = ln.state == kNotify && !same && ln.c2 == 1;
  const uint32_t nmask1 = __ballot_sync(0xffffffffu, push1);
  const uint32_t nmask2 = __ballot_sync(0xffffffffu, push2);
  if (nmask1 | nmask2) {
    const int leader = __ffs(nmask1 | nmask2) - 1;
    uint32_t base = 0;
    if (lane == static_cast<uint32_t>(leader)) base = atomicAdd(q.ctl + 1, __popc(nmask1) + __popc(nmask2));
    base = __shfl_sync(0xffffffffu, base, leader);
    const PipeSoup &sp = b.soups[ln.si];
    const uint32_t next = sp.task_base + (ln.e + 1) * sp.npairs;
    if (push1) st_release_u32(q.queue + base + __popc(nmask1 & lt_mask), next + (ln.j1 >> 1) + 1);
    if (push2)
      st_release_u32(q.queue + base + __popc(nmask1) + __popc(nmask2 & lt_mask),
                     next + (ln.j2 >> 1) + 1);
  }
  if (ln.state == kNotify) ln.state = kIdle;
  return progressed;
}

// A warp serves queue q until every lane has claimed past its last task.
template <int L>
__device__ __forceinline__ void serve(const PipeCtx &b, const PipeQueue &q,
                                      const uint8_t *__restrict__ optab,
                                      const uint8_t *__restrict__ cmdflag, const LaneBytes t,
                                      const LaneBytes stk, const LaneNp np, uint32_t lane,
                                      uint32_t slot_ctr) {
  Lane ln;
  ln.state = kIdle;
  ln.slot = ln.task = ln.e = ln.k = ln.p1 = ln.p2 = ln.qv = 0;
  ln.poll_gap = 1;
  ln.poll_in = ln.err = ln.j1 = ln.j2 = ln.c1 = ln.c2 = ln.visits = 0;
  ln.si = 0;
  ln.qp = ln.t_wait = 0;
  ln.dirty = ln.evaluated = ln.has_next = false;
  ln.mm = make_uint4(0, 0, 0, 0);
  LaneMachine<L> m;
  while (true) {
    const bool progressed = iterate<L>(b, q, ln, m, t, stk, np, optab, cmdflag, lane, slot_ctr);
    if (__all_sync(0xffffffffu, ln.state == kExhausted)) return;
    if (!__any_sync(0xffffffffu, progressed)) __nanosleep(200);
  }
}

// Shared memory of a pipelined launch: the tape and second areas, the BFF
// next-command arrays (BFF family only), the op and command tables, then the
// soup descriptors.
template <int L>
__host__ __device__ constexpr size_t pipeline_np_bytes() {
  return L <= kBffSelfmove ? size_t(kNpBytes) : 0;
}

template <int L>
size_t pipeline_smem_bytes(int n_soups) {
  return 2 * kGroups * kGroupBytes + pipeline_np_bytes<L>() + 512 +
         size_t(n_soups) * sizeof(PipeSoup);
}

// The persistent kernel of a pipelined launch over soups of language L.  The
// BFF family's larger shared-memory footprint allows 3 blocks per SM, the
// others 4; the register budget follows.
template <int L>
__global__ void __launch_bounds__(kThreads, (L <= kBffSelfmove) ? 3 : 4)
    pipeline_kernel(const __grid_constant__ PipeBatch pb) {
  extern __shared__ __align__(16) uint8_t smem[];
  uint16_t *npa = reinterpret_cast<uint16_t *>(smem + 2 * kGroups * kGroupBytes);
  uint8_t *optab = smem + 2 * kGroups * kGroupBytes + pipeline_np_bytes<L>();
  uint8_t *cmdflag = optab + 256;
  PipeSoup *soups = reinterpret_cast<PipeSoup *>(optab + 512);
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  if (LangTraits<L>::kNeedsTable) {
    for (uint32_t c = tid; c < 256; c += kThreads) {
      optab[c] = op_of(L, c);
      cmdflag[c] = op_of(L, c) < kNull;
    }
  }
  {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(pb.soups);
    uint32_t *dst = reinterpret_cast<uint32_t *>(soups);
    const uint32_t words = pb.n_soups * sizeof(PipeSoup) / 4;
    for (uint32_t i = tid; i < words; i += kThreads) dst[i] = src[i];
  }
  __syncthreads();  // tables and descriptors are read-only from here on
  const LaneBytes t{smem, lane_base(tid)};
  const LaneBytes stk{smem + kGroups * kGroupBytes, lane_base(tid)};
  const uint32_t warp = blockIdx.x * (kThreads / 32) + (tid >> 5);
  const LaneNp np{L <= kBffSelfmove ? npa : nullptr, tid};
  const PipeCtx b{soups, pb.error, pb.wait_limit_ns, pb.tune};
  const PipeQueue q = pb.queue;
  serve<L>(b, q, optab, cmdflag, t, stk, np, lane, warp % kCountSlots);
}

template <int L>
int launch_pipeline_t(const PipeBatch &b, uint64_t total_pairs, uint32_t lanes_per_pair64,
                      int device, cudaStream_t stream) {
  static std::atomic<int> sms_cache[64];  // (zero-initialised: static storage)
  const size_t smem_max = pipeline_smem_bytes<L>(kMaxPipeSoups);
  if (sms_cache[device & 63].load() == 0) {
    CUBFF_CUDA_TRY(cudaFuncSetAttribute(pipeline_kernel<L>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem_max)));
    int sms = 0;
    CUBFF_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    sms_cache[device & 63].store(sms);
  }
  const size_t smem = pipeline_smem_bytes<L>(b.n_soups);
  int per_sm = 0;
  CUBFF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pipeline_kernel<L>,
                                                               kThreads, smem));
  const uint64_t resident = uint64_t(std::max(1, per_sm)) * sms_cache[device & 63].load();
  // Lanes in flight: enough to keep the SMs busy, few enough that most held
  // pairs are ready (a lane holding a pair of a later epoch only polls).
  // lanes_per_pair64 (x1/64) is tunable; the default keeps half an epoch of
  // pairs in flight.
  uint64_t want = (total_pairs * uint64_t(lanes_per_pair64 ? lanes_per_pair64 : 32)) / 64;
  want = std::max<uint64_t>(want, kThreads);
  const uint64_t blocks = (want + kThreads - 1) / kThreads;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(blocks, resident));
  pipeline_kernel<L><<<grid, kThreads, smem, stream>>>(b);
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
}

}  // namespace

uint64_t pipeline_wait_limit_ns() { return g_wait_limit_ns.load(); }

namespace {
uint32_t env_u32(const char *name, uint32_t dflt, uint32_t lo, uint32_t hi) {
  const char *v = std::getenv(name);
  if (!v || !*v) return dflt;
  const long x = std::strtol(v, nullptr, 10);
  return x < long(lo) ? lo : x > long(hi) ? hi : static_cast<uint32_t>(x);
}
}  // namespace

// Default launch shape: half an epoch of pairs in flight, 64 steps per visit,
// claims by warps with at least 20 idle lanes, pairs past their first visit
// kept without new warp-mates.
cubff_tuning default_shape() {
  static const cubff_tuning t = {env_u32("CUBFF_LANES_PER_PAIR64", 32, 1, 64),
                                 env_u32("CUBFF_STEPS_PER_VISIT", 64, 1, 4096),
                                 env_u32("CUBFF_CLAIM_MIN", 20, 1, 32),
                                 env_u32("CUBFF_LONG_VISITS", 1, 0, 1u << 20),
                                 env_u32("CUBFF_FIRST_VISIT_STEPS", 64, 1, 4096)};
  return t;
}

bool valid_shape(const cubff_tuning &t) {
  return t.lanes_per_pair64 >= 1 && t.lanes_per_pair64 <= 64 && t.steps_per_visit >= 1 &&
         t.steps_per_visit <= 4096 && t.claim_min >= 1 && t.claim_min <= 32 &&
         t.first_visit_steps >= 1 && t.first_visit_steps <= 4096;
}

PipeTuning pipe_tuning(const cubff_tuning &t) {
  return PipeTuning{t.steps_per_visit, t.claim_min,
                    t.long_visits ? t.long_visits : 0xffffffffu, t.first_visit_steps};
}

int launch_pipeline(const PipeBatch &b, uint64_t total_pairs, uint32_t lanes_per_pair64,
                    int device, cudaStream_t stream) {
  if (b.n_soups <= 0 || total_pairs == 0) return CUBFF_OK;
  if (b.n_soups > kMaxPipeSoups)
    return set_error(CUBFF_EINVAL, "pipeline: %d soups over the limit of %d", b.n_soups,
                     kMaxPipeSoups);
  const uint32_t tpp = lanes_per_pair64;
  switch (b.queue.lang) {
    case kBff: return launch_pipeline_t<kBff>(b, total_pairs, tpp, device, stream);
    case kBffNoheads: return launch_pipeline_t<kBffNoheads>(b, total_pairs, tpp, device, stream);
    case kBffNoheads4bit: return launch_pipeline_t<kBffNoheads4bit>(b, total_pairs, tpp, device, stream);
    case kBffPerm: return launch_pipeline_t<kBffPerm>(b, total_pairs, tpp, device, stream);
    case kBff8: return launch_pipeline_t<kBff8>(b, total_pairs, tpp, device, stream);
    case kBff8Noheads: return launch_pipeline_t<kBff8Noheads>(b, total_pairs, tpp, device, stream);
    case kBffSelfmove: return launch_pipeline_t<kBffSelfmove>(b, total_pairs, tpp, device, stream);
    case kForth: return launch_pipeline_t<kForth>(b, total_pairs, tpp, device, stream);
    case kForthcopy: return launch_pipeline_t<kForthcopy>(b, total_pairs, tpp, device, stream);
    case kForthtrivial: return launch_pipeline_t<kForthtrivial>(b, total_pairs, tpp, device, stream);
    case kForthtrivialReset:
      return launch_pipeline_t<kForthtrivialReset>(b, total_pairs, tpp, device, stream);
    case kSubleq: return launch_pipeline_t<kSubleq>(b, total_pairs, tpp, device, stream);
    case kRsubleq4: return launch_pipeline_t<kRsubleq4>(b, total_pairs, tpp, device, stream);
  }
  return set_error(CUBFF_ENOTFOUND, "unknown language id %d", b.queue.lang);
}

int launch_mutation_masks(uint64_t s0, uint64_t e0, uint32_t n_epochs, uint64_t n, uint32_t prob,
                          uint4 *out, cudaStream_t stream) {
  const uint64_t words = (n / 2) * n_epochs * 4;
  if (words == 0) return CUBFF_OK;
  mutation_mask_kernel<<<static_cast<unsigned>((words + 255) / 256), 256, 0, stream>>>(
      s0, e0, n / 2, words, n, prob, reinterpret_cast<uint32_t *>(out));
  CUBFF_CUDA_TRY(cudaGetLastError());
  return CUBFF_OK;
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
  return cubff_run_epochs_tuned(lang, d_programs, d_shuf_idx, d_num_indices, params_seed,
                                first_epoch, n_epochs, mutation_prob, num_programs, d_counts,
                                d_workspace, workspace_bytes, nullptr, stream);
}

extern "C" void cubff_default_tuning(cubff_tuning *out) {
  if (out) *out = cubff::default_shape();
}

extern "C" int cubff_run_epochs_tuned(int lang, uint8_t *d_programs, const uint32_t *d_shuf_idx,
                                      const uint64_t *d_num_indices, uint64_t params_seed,
                                      uint64_t first_epoch, uint32_t n_epochs,
                                      uint32_t mutation_prob, uint64_t num_programs,
                                      unsigned long long *d_counts, void *d_workspace,
                                      size_t workspace_bytes, const cubff_tuning *tuning,
                                      void *stream) {
  using namespace cubff;
  const cubff_tuning shape = tuning ? *tuning : default_shape();
  if (!valid_shape(shape)) return set_error(CUBFF_EINVAL, "run_epochs: launch shape out of range");
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
  if ((num_programs / 2) * uint64_t(n_epochs) >= (1ull << 31))
    return set_error(CUBFF_EINVAL, "run_epochs: num_programs/2 * n_epochs must be < 2^31");
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
  PipeBatch b;
  PipeSoup &sp = b.soups[0];
  sp.soup = d_programs;
  sp.perm = d_shuf_idx;
  sp.inv = w.inv;
  sp.mutmask = w.mutmask;
  sp.readycnt = w.readycnt;
  sp.num_indices = d_num_indices;
  sp.ops = w.counters;
  sp.n = n;
  sp.s0 = s0;
  sp.e0 = first_epoch;
  sp.npairs = static_cast<uint32_t>(P);
  sp.mutation_prob = mutation_prob;
  sp.task_base = 0;
  sp.init_base = 0;
  sp.lang = lang;
  sp.n_epochs = n_epochs;
  PipeQueue &q = b.queue;
  q.queue = w.queue;
  q.ctl = w.ctl;
  q.total = static_cast<uint32_t>(P * n_epochs);
  q.initial = static_cast<uint32_t>(P);
  q.first_soup = 0;
  q.n_soups = 1;
  q.lang = lang;
  b.n_soups = 1;
  b.error = reinterpret_cast<int *>(w.ctl + 2);
  b.wait_limit_ns = pipeline_wait_limit_ns();
  b.tune = pipe_tuning(shape);
  CUBFF_TRY(launch_pipeline(b, P, shape.lanes_per_pair64, dev, st));
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
  if (err == 2) return set_error(CUBFF_EDEVICE, "run_epochs: a ready-queue entry was out of range");
  if (err) return set_error(CUBFF_ETIMEDOUT, "run_epochs: a pipelined wait timed out");
  return CUBFF_OK;
}

extern "C" int cubff_set_wait_limit_ns(uint64_t ns, uint64_t *previous) {
  using namespace cubff;
  if (ns == 0) return set_error(CUBFF_EINVAL, "set_wait_limit_ns: the limit must be > 0");
  const uint64_t old = g_wait_limit_ns.exchange(ns);
  if (previous) *previous = old;
  return CUBFF_OK;
}
