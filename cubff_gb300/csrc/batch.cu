// batch.cu — pipelined runs of one or more soups (cubff_soup_run,
// cubff_batch_run).
//
// The soups of a run (any languages, sizes, mutation rates and pairing
// modes) are split into launch groups: one language, at most kMaxPipeSoups
// soups each.  A group advances in rounds; a round is one persistent
// pipeline launch (pipeline.cu) covering the next segment of epochs of every
// soup in the group.  A soup's segment ends where its cached pairings end,
// at a reset epoch (a reset rewrites every program at once,
// common_language.h:590-595), at the end of its op-counter chunk, or at the
// end of the run.  Groups run on streams of their own, forked from and joined
// back to the engine stream, so the launches of different languages overlap;
// the host enqueues all rounds without waiting, except to read the op
// counters back every kCounterChunk epochs and for host-computed (pattern)
// pairings.
#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "engine_impl.h"
#include "internal.h"

namespace cubff {

// Keeps queue ids (task + 1, uint32) and the queue heads, which overshoot the
// task count by at most 32 per warp, clear of 2^32.
static constexpr uint64_t kMaxTasksPerLaunch = (1ull << 31) - (1ull << 22);

}  // namespace cubff

using namespace cubff;

int cubff_engine::reserve_pipe(size_t groups, size_t entries) {
  while (streams.size() < groups) {
    cudaStream_t s = nullptr;
    CUBFF_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    streams.push_back(s);
  }
  while (events.size() < groups + 1) {
    cudaEvent_t e = nullptr;
    CUBFF_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    events.push_back(e);
  }
  if (groups > ctl_groups) {
    if (d_ctl) cudaFree(d_ctl);
    if (h_ctl) cudaFreeHost(h_ctl);
    d_ctl = h_ctl = nullptr;
    ctl_groups = 0;
    CUBFF_CUDA_TRY(cudaMalloc(&d_ctl, groups * 4 * sizeof(uint32_t)));
    CUBFF_CUDA_TRY(cudaMallocHost(&h_ctl, groups * 4 * sizeof(uint32_t)));
    ctl_groups = groups;
  }
  if (entries > queue_cap) {
    if (d_queue) cudaFree(d_queue);
    d_queue = nullptr;
    queue_cap = 0;
    CUBFF_CUDA_TRY(cudaMalloc(&d_queue, entries * sizeof(uint32_t)));
    // On the engine's stream: the pipelined kernels run on non-blocking
    // streams, which a memset on the legacy default stream does not order.
    CUBFF_CUDA_TRY(cudaMemsetAsync(d_queue, 0, entries * sizeof(uint32_t), stream));
    queue_cap = entries;
  }
  return CUBFF_OK;
}

void cubff_engine::release_pipe() {
  for (cudaStream_t s : streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : events) cudaEventDestroy(e);
  streams.clear();
  events.clear();
  if (d_queue) cudaFree(d_queue);
  if (d_ctl) cudaFree(d_ctl);
  if (h_ctl) cudaFreeHost(h_ctl);
  d_queue = nullptr;
  d_ctl = h_ctl = nullptr;
  queue_cap = ctl_groups = 0;
}

namespace cubff {
namespace {

struct Group {
  int lang;
  std::vector<int> members;  // indices into the run's soups
  cudaStream_t st;
  size_t qoff;               // first entry of the group's ready queue in d_queue
  uint64_t programs = 0;     // summed over the members (the launch-shape key)
};

// Per-soup progress of a run.
struct Progress {
  uint64_t done = 0;   // epochs of this run enqueued
  uint64_t cbase = 0;  // run epoch of counter row 0
  uint32_t seg = 0;    // epochs of the round being built
};

}  // namespace

// Reads back and reduces the op counters of every soup of the run, and the
// groups' error flags.  The groups' streams must be idle (synchronised).
static int read_counters(cubff_soup *const *soups, const std::vector<Group> &groups,
                         std::vector<Progress> &pr, uint64_t *const *ops, uint64_t *const *raw,
                         const uint32_t *h_ctl, uint32_t *fault) {
  for (const Group &g : groups) {
    *fault = std::max(*fault, h_ctl[4 * (&g - groups.data()) + 2]);
    for (int i : g.members) {
      const uint64_t rows = pr[i].done - pr[i].cbase;
      const unsigned long long *h = soups[i]->h_counters;
      for (uint64_t q = 0; q < rows; q++) {
        uint64_t o = 0, r = 0;
        for (int sl = 0; sl < kPipeCountSlots; sl++) {
          o += h[(q * kPipeCountSlots + sl) * 2];
          r += h[(q * kPipeCountSlots + sl) * 2 + 1];
        }
        if (ops && ops[i]) ops[i][pr[i].cbase + q] = o;
        if (raw && raw[i]) raw[i][pr[i].cbase + q] = r;
      }
    }
  }
  return CUBFF_OK;
}

// Enqueues the copies that read_counters consumes, on each group's stream.
static int copy_counters(cubff_soup *const *soups, const std::vector<Group> &groups,
                         const std::vector<Progress> &pr, const cubff_engine *eng) {
  for (size_t gi = 0; gi < groups.size(); gi++) {
    const Group &g = groups[gi];
    for (int i : g.members) {
      const uint64_t rows = pr[i].done - pr[i].cbase;
      if (rows)
        CUBFF_CUDA_TRY(cudaMemcpyAsync(soups[i]->h_counters, soups[i]->d_counters,
                                       rows * kPipeCountSlots * 2 * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, g.st));
    }
    CUBFF_CUDA_TRY(cudaMemcpyAsync(eng->h_ctl + 4 * gi, eng->d_ctl + 4 * gi, 4 * sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, g.st));
  }
  return CUBFF_OK;
}

int run_soups(cubff_engine *eng, cubff_soup *const *soups, int n_soups, uint64_t n_epochs,
              uint64_t *const *ops, uint64_t *const *raw, uint64_t *const *ni,
              const uint64_t *epochs_each) {
  if (n_soups == 0) return CUBFF_OK;
  // Epochs soup i advances: its own count, or n_epochs for all.
  auto want = [&](int i) { return epochs_each ? epochs_each[i] : n_epochs; };
  bool any_work = false;
  for (int i = 0; i < n_soups; i++) any_work |= want(i) > 0;
  if (!any_work) return CUBFF_OK;
  constexpr uint64_t kChunk = cubff_soup::kCounterChunk;
  for (int i = 0; i < n_soups; i++) CUBFF_TRY(soups[i]->ensure_buffers());

  // Launch groups: by language, at most kMaxPipeSoups soups each.
  std::vector<int> order(n_soups);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return soups[a]->p.lang < soups[b]->p.lang; });
  std::vector<Group> groups;
  size_t entries = 0;
  for (int i : order) {
    if (groups.empty() || groups.back().lang != soups[i]->p.lang ||
        groups.back().members.size() == size_t(kMaxPipeSoups))
      groups.push_back(Group{soups[i]->p.lang, {}, nullptr, entries, 0});
    groups.back().members.push_back(i);
    groups.back().programs += soups[i]->p.num_programs;
    entries += size_t(soups[i]->batch) * (soups[i]->p.num_programs / 2);
  }
  const size_t G = groups.size();
  CUBFF_TRY(eng->reserve_pipe(G, entries));
  cudaStream_t main = eng->stream;
  for (size_t g = 0; g < G; g++) groups[g].st = G == 1 ? main : eng->streams[g];

  // State left behind by a launch that gave up.
  if (eng->dirty) {
    CUBFF_CUDA_TRY(cudaMemsetAsync(eng->d_queue, 0, eng->queue_cap * sizeof(uint32_t), main));
    eng->dirty = false;
  }
  for (int i = 0; i < n_soups; i++) {
    cubff_soup *s = soups[i];
    if (s->dirty) {
      CUBFF_CUDA_TRY(cudaMemsetAsync(s->d_readycnt, 0,
                                     size_t(s->batch) * (s->p.num_programs / 2) * sizeof(uint32_t),
                                     main));
      s->dirty = false;
    }
  }
  CUBFF_CUDA_TRY(cudaMemsetAsync(eng->d_ctl, 0, G * 4 * sizeof(uint32_t), main));
  if (G > 1) {
    CUBFF_CUDA_TRY(cudaEventRecord(eng->events[0], main));
    for (size_t g = 0; g < G; g++) CUBFF_CUDA_TRY(cudaStreamWaitEvent(groups[g].st, eng->events[0], 0));
  }

  std::vector<Progress> pr(n_soups);
  for (const Group &g : groups) {
    for (int i : g.members) {
      cubff_soup *s = soups[i];
      if (want(i) == 0) continue;
      if (s->pending_reset) {
        CUBFF_TRY(s->apply_reset(g.st));
        s->pending_reset = false;
      }
      const uint64_t first_rows = std::min<uint64_t>(want(i), kChunk);
      CUBFF_CUDA_TRY(cudaMemsetAsync(s->d_counters, 0,
                                     first_rows * kPipeCountSlots * 2 * sizeof(unsigned long long),
                                     g.st));
    }
  }

  std::unique_ptr<PipeBatch> b(new PipeBatch);
  uint32_t fault = 0;  // the launches' error flag: 1 a wait timed out, 2 a bad queue entry
  while (true) {
    // A soup whose counter chunk is full: read every soup's counters back.
    bool flush = false;
    for (int i = 0; i < n_soups; i++)
      flush |= pr[i].done < want(i) && pr[i].done - pr[i].cbase == kChunk;
    if (flush) {
      CUBFF_TRY(copy_counters(soups, groups, pr, eng));
      for (const Group &g : groups) CUBFF_CUDA_TRY(cudaStreamSynchronize(g.st));
      CUBFF_TRY(read_counters(soups, groups, pr, ops, raw, eng->h_ctl, &fault));
      if (fault) break;
      for (const Group &g : groups) {
        for (int i : g.members) {
          pr[i].cbase = pr[i].done;
          const uint64_t rows = std::min<uint64_t>(want(i) - pr[i].done, kChunk);
          if (rows)
            CUBFF_CUDA_TRY(cudaMemsetAsync(soups[i]->d_counters, 0,
                                           rows * kPipeCountSlots * 2 * sizeof(unsigned long long),
                                           g.st));
        }
      }
    }

    bool any = false;
    for (size_t gi = 0; gi < G; gi++) {
      Group &g = groups[gi];
      PipeBatch &pb = *b;
      pb.n_soups = 0;
      uint64_t tasks = 0, pairs = 0;
      uint32_t initial = 0;
      for (int i : g.members) {
        cubff_soup *s = soups[i];
        Progress &p = pr[i];
        p.seg = 0;
        if (p.done >= want(i)) continue;
        const uint64_t n = s->p.num_programs, P = n / 2;
        const uint64_t e = s->epoch + p.done;
        if (s->perm_count == 0 || e < s->perm_first || e >= s->perm_first + s->perm_count)
          CUBFF_TRY(s->fill_pairing(e, static_cast<uint32_t>(std::min<uint64_t>(s->batch, want(i) - p.done)),
                                    g.st));
        uint64_t seg = std::min<uint64_t>(s->perm_first + s->perm_count - e, want(i) - p.done);
        seg = std::min<uint64_t>(seg, p.cbase + kChunk - p.done);
        if (s->p.reset_interval) {
          const uint64_t r = e + (s->p.reset_interval - e % s->p.reset_interval) % s->p.reset_interval;
          seg = std::min<uint64_t>(seg, r - e + 1);
        }
        if (tasks + P * seg > kMaxTasksPerLaunch) {
          if (pb.n_soups > 0) continue;  // runs in a later round
          seg = std::max<uint64_t>(1, kMaxTasksPerLaunch / P);
        }
        const uint64_t slot = e - s->perm_first;
        PipeSoup &d = pb.soups[pb.n_soups++];
        d.soup = s->d_soup;
        d.perm = s->d_perm + slot * n;
        d.inv = s->d_inv + slot * n;
        d.mutmask = s->d_mutmask + slot * P;
        d.readycnt = s->d_readycnt;
        d.num_indices = s->p.pairing == CUBFF_PAIR_PATTERN ? s->d_num_indices + slot : nullptr;
        d.ops = s->d_counters + (p.done - p.cbase) * kPipeCountSlots * 2;
        d.n = n;
        d.s0 = s->s0;
        d.e0 = e;
        d.npairs = static_cast<uint32_t>(P);
        d.mutation_prob = s->p.mutation_prob;
        d.task_base = static_cast<uint32_t>(tasks);
        d.init_base = initial;
        d.lang = s->p.lang;
        d.n_epochs = static_cast<uint32_t>(seg);
        tasks += P * seg;
        initial += static_cast<uint32_t>(P);
        pairs += P;
        p.seg = static_cast<uint32_t>(seg);
        if (ni && ni[i]) {
          for (uint64_t q = 0; q < seg; q++)
            ni[i][p.done + q] = s->p.pairing == CUBFF_PAIR_PATTERN ? s->h_pat_ni[slot + q] : P;
        }
      }
      if (pb.n_soups == 0) continue;
      any = true;
      PipeQueue &q = pb.queue;
      q.queue = eng->d_queue + g.qoff;
      q.ctl = eng->d_ctl + 4 * gi;
      q.total = static_cast<uint32_t>(tasks);
      q.initial = initial;
      q.first_soup = 0;
      q.n_soups = static_cast<uint32_t>(pb.n_soups);
      q.lang = g.lang;
      pb.error = reinterpret_cast<int *>(eng->d_ctl + 4 * gi + 2);
      pb.wait_limit_ns = pipeline_wait_limit_ns();
      const cubff_tuning shape = eng->shape_for(g.lang, g.programs, static_cast<uint32_t>(g.members.size()));
      pb.tune = pipe_tuning(shape);
      CUBFF_CUDA_TRY(cudaMemsetAsync(q.ctl, 0, 2 * sizeof(uint32_t), g.st));  // head, tail
      CUBFF_TRY(launch_pipeline(pb, pairs, shape.lanes_per_pair64, eng->device, g.st));
      for (int i : g.members) {
        cubff_soup *s = soups[i];
        Progress &p = pr[i];
        if (p.seg == 0) continue;
        const uint64_t last = s->epoch + p.done + p.seg - 1;
        p.done += p.seg;
        if (s->p.reset_interval && last % s->p.reset_interval == 0) {
          if (p.done == want(i)) s->pending_reset = true;
          else CUBFF_TRY(s->apply_reset(g.st));
        }
      }
    }
    if (!any) break;
  }

  if (!fault) {
    CUBFF_TRY(copy_counters(soups, groups, pr, eng));
    for (const Group &g : groups) CUBFF_CUDA_TRY(cudaStreamSynchronize(g.st));
    CUBFF_TRY(read_counters(soups, groups, pr, ops, raw, eng->h_ctl, &fault));
  }
  if (G > 1) {
    for (size_t g = 0; g < G; g++) {
      CUBFF_CUDA_TRY(cudaEventRecord(eng->events[1 + g], groups[g].st));
      CUBFF_CUDA_TRY(cudaStreamWaitEvent(main, eng->events[1 + g], 0));
    }
  }
  for (int i = 0; i < n_soups; i++) soups[i]->epoch += pr[i].done;
  if (fault) {
    eng->dirty = true;
    for (int i = 0; i < n_soups; i++) soups[i]->dirty = true;
    if (fault == 2)
      return set_error(CUBFF_EDEVICE,
                       "a ready-queue entry was out of range; the soups' state is invalid");
    return set_error(CUBFF_ETIMEDOUT,
                     "a pipelined epoch wait timed out; the soups' state is invalid");
  }
  return CUBFF_OK;
}

}  // namespace cubff

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
  std::vector<uint64_t *> outs(n_soups);
  for (int s = 0; s < n_soups; s++) outs[s] = ops ? ops + size_t(s) * n_epochs : nullptr;
  return run_soups(eng, soups, n_soups, n_epochs, outs.data(), nullptr, nullptr);
}
