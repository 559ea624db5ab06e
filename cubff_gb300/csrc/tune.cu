// tune.cu — the launch-shape tuner (cubff_engine_tune) and the engine's cache
// of tuned shapes.
//
// The reference launches every epoch with one fixed shape: ceil(N/64)
// blocks of 32 threads, one thread per pair (common_language.h:348,
// :490-493).  The pipelined launch here has five knobs (cubff_tuning): lanes
// in flight per 64 pairs, steps per visit (the first, and the later ones),
// the claim threshold of busy warps and the visit count after which a pair
// keeps its warp from claiming.  The best values depend on the language
// (step cost, how long pairs run), on the number of programs in the launch
// and on how many soups share it, so the engine keeps one shape per
// (language, log2 programs, log2 soups) key.
//
// Tuning runs a few epochs of scratch copies of the caller's soups under
// candidate shapes (coordinate descent from the default: each knob in turn
// over a short list of values, the others fixed; two passes), per language,
// timed on the host around the synchronous run.  Every candidate must give
// the same op counts (shapes change timing only); a disagreement is an error.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "engine_impl.h"
#include "internal.h"

using namespace cubff;

namespace {

uint32_t log2_bucket(uint64_t x) {
  uint32_t b = 0;
  while (x > 1) {
    x >>= 1;
    b++;
  }
  return b;
}

// A scratch copy of a soup: same parameters and interaction lists, bytes and
// epoch restored from the original before every trial.
struct Clone {
  cubff_soup *orig = nullptr;
  cubff_soup *copy = nullptr;
};

int restore(Clone &c) {
  cubff_soup *o = c.orig, *s = c.copy;
  CUBFF_CUDA_TRY(cudaMemcpyAsync(s->d_soup, o->d_soup, o->p.num_programs * kTape,
                                 cudaMemcpyDeviceToDevice, s->eng->stream));
  s->epoch = o->epoch;
  s->reset_index = o->reset_index;
  s->pending_reset = o->pending_reset;
  return CUBFF_OK;
}

struct Trial {
  double seconds = 0;
  std::vector<uint64_t> ops;  // every soup's op counts, epoch by epoch
};

int run_trial(cubff_engine *eng, std::vector<Clone> &clones, uint32_t epochs,
              const cubff_tuning &shape, Trial *out) {
  for (Clone &c : clones) CUBFF_TRY(restore(c));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(eng->stream));
  std::vector<cubff_soup *> soups;
  std::vector<uint64_t> ops(clones.size() * epochs, 0);
  std::vector<uint64_t *> outs;
  for (size_t i = 0; i < clones.size(); i++) {
    soups.push_back(clones[i].copy);
    outs.push_back(ops.data() + i * epochs);
  }
  eng->forced = &shape;
  const auto t0 = std::chrono::steady_clock::now();
  const int st = run_soups(eng, soups.data(), static_cast<int>(soups.size()), epochs, outs.data(),
                           nullptr, nullptr);
  const auto t1 = std::chrono::steady_clock::now();
  eng->forced = nullptr;
  CUBFF_TRY(st);
  out->seconds = std::chrono::duration<double>(t1 - t0).count();
  out->ops = std::move(ops);
  return CUBFF_OK;
}

bool same_shape(const cubff_tuning &a, const cubff_tuning &b) {
  return std::memcmp(&a, &b, sizeof(a)) == 0;
}

// Coordinate descent for the clones of one language.
int tune_language(cubff_engine *eng, std::vector<Clone> &clones, uint32_t epochs,
                  cubff_tuning *best_out) {
  static const uint32_t kLanes[] = {16, 24, 32, 48, 64};
  static const uint32_t kSteps[] = {16, 32, 64, 128, 256};
  static const uint32_t kClaim[] = {8, 14, 20, 26, 32};
  static const uint32_t kLong[] = {0, 1, 2, 4, 8};
  static const uint32_t kFirst[] = {4, 8, 16, 32, 64};
  cubff_tuning best = default_shape();
  Trial warm, ref;
  CUBFF_TRY(run_trial(eng, clones, epochs, best, &warm));  // pairings cached, caches warm
  CUBFF_TRY(run_trial(eng, clones, epochs, best, &ref));
  double best_s = std::min(warm.seconds, ref.seconds);
  auto time_of = [&](const cubff_tuning &cand, double *sec) -> int {
    Trial a, b;
    CUBFF_TRY(run_trial(eng, clones, epochs, cand, &a));
    CUBFF_TRY(run_trial(eng, clones, epochs, cand, &b));
    if (a.ops != ref.ops || b.ops != ref.ops)
      return set_error(CUBFF_EDEVICE, "tune: launch shapes gave different op counts");
    *sec = std::min(a.seconds, b.seconds);
    return CUBFF_OK;
  };
  for (int pass = 0; pass < 2; pass++) {
    for (int knob = 0; knob < 5; knob++) {
      const uint32_t *vals = knob == 0 ? kLanes : knob == 1 ? kSteps : knob == 2 ? kClaim
                             : knob == 3 ? kLong : kFirst;
      cubff_tuning round_best = best;
      for (int v = 0; v < 5; v++) {
        cubff_tuning cand = best;
        uint32_t *field = knob == 0 ? &cand.lanes_per_pair64
                          : knob == 1 ? &cand.steps_per_visit
                          : knob == 2 ? &cand.claim_min
                          : knob == 3 ? &cand.long_visits
                                      : &cand.first_visit_steps;
        *field = vals[v];
        if (same_shape(cand, best)) continue;
        double sec = 0;
        CUBFF_TRY(time_of(cand, &sec));
        if (sec < best_s) {
          best_s = sec;
          round_best = cand;
        }
      }
      best = round_best;
    }
  }
  *best_out = best;
  return CUBFF_OK;
}

}  // namespace

uint64_t cubff_engine::shape_key(int lang, uint64_t group_programs, uint32_t group_soups) {
  return uint64_t(uint32_t(lang)) | uint64_t(log2_bucket(group_programs)) << 8 |
         uint64_t(log2_bucket(group_soups)) << 16;
}

cubff_tuning cubff_engine::shape_for(int lang, uint64_t group_programs, uint32_t group_soups) const {
  if (forced) return *forced;
  auto it = shapes.find(shape_key(lang, group_programs, group_soups));
  return it != shapes.end() ? it->second : default_shape();
}

extern "C" {

int cubff_engine_get_tuning(cubff_engine *eng, int lang, uint64_t group_programs,
                            uint32_t group_soups, cubff_tuning *out) {
  if (!eng || !out) return set_error(CUBFF_EINVAL, "get_tuning: null argument");
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  *out = eng->shape_for(lang, group_programs, group_soups);
  return CUBFF_OK;
}

int cubff_engine_set_tuning(cubff_engine *eng, int lang, uint64_t group_programs,
                            uint32_t group_soups, const cubff_tuning *t) {
  if (!eng || !t) return set_error(CUBFF_EINVAL, "set_tuning: null argument");
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  if (!valid_shape(*t)) return set_error(CUBFF_EINVAL, "set_tuning: knob out of range");
  eng->shapes[cubff_engine::shape_key(lang, group_programs, group_soups)] = *t;
  return CUBFF_OK;
}

int cubff_engine_tune(cubff_engine *eng, cubff_soup **soups, int n_soups, uint32_t trial_epochs,
                      cubff_tuning *chosen) {
  if (!eng || !soups || n_soups <= 0) return set_error(CUBFF_EINVAL, "tune: bad arguments");
  for (int i = 0; i < n_soups; i++) {
    if (!soups[i] || soups[i]->eng != eng)
      return set_error(CUBFF_EINVAL, "tune: soup %d is null or on another engine", i);
    if (soups[i]->p.pairing == CUBFF_PAIR_PATTERN && soups[i]->pat_offs.empty())
      return set_error(CUBFF_EINVAL, "tune: soup %d needs its interaction lists", i);
  }
  if (trial_epochs == 0) trial_epochs = 16;
  CUBFF_CUDA_TRY(cudaSetDevice(eng->device));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(eng->stream));
  int status = CUBFF_OK;
  for (int lang = 0; lang < kNumLangs && status == CUBFF_OK; lang++) {
    std::vector<Clone> clones;
    for (int i = 0; i < n_soups && status == CUBFF_OK; i++) {
      if (soups[i]->p.lang != lang) continue;
      Clone c;
      c.orig = soups[i];
      status = cubff_soup_create(eng, &soups[i]->p, &c.copy);
      if (status == CUBFF_OK && soups[i]->p.pairing == CUBFF_PAIR_PATTERN)
        status = cubff_soup_set_pattern(c.copy, soups[i]->pat_offs.data(),
                                        soups[i]->pat_tgts.data());
      if (c.copy) clones.push_back(c);
    }
    cubff_tuning best{};
    if (status == CUBFF_OK && !clones.empty()) status = tune_language(eng, clones, trial_epochs, &best);
    if (status == CUBFF_OK && !clones.empty()) {
      // The launch groups run_soups forms for these soups: runs of at most
      // kMaxPipeSoups of them, in order.
      for (size_t g0 = 0; g0 < clones.size(); g0 += kMaxPipeSoups) {
        const size_t g1 = std::min(clones.size(), g0 + kMaxPipeSoups);
        uint64_t programs = 0;
        for (size_t i = g0; i < g1; i++) programs += clones[i].orig->p.num_programs;
        eng->shapes[cubff_engine::shape_key(lang, programs, static_cast<uint32_t>(g1 - g0))] = best;
      }
    }
    for (Clone &c : clones) cubff_soup_destroy(c.copy);
  }
  if (status != CUBFF_OK) return status;
  if (chosen) {
    // The shape each soup's launch group now uses, as run_soups groups them.
    for (int lang = 0; lang < kNumLangs; lang++) {
      std::vector<int> idx;
      for (int i = 0; i < n_soups; i++)
        if (soups[i]->p.lang == lang) idx.push_back(i);
      for (size_t g0 = 0; g0 < idx.size(); g0 += kMaxPipeSoups) {
        const size_t g1 = std::min(idx.size(), g0 + kMaxPipeSoups);
        uint64_t programs = 0;
        for (size_t q = g0; q < g1; q++) programs += soups[idx[q]]->p.num_programs;
        const cubff_tuning t = eng->shape_for(lang, programs, static_cast<uint32_t>(g1 - g0));
        for (size_t q = g0; q < g1; q++) chosen[idx[q]] = t;
      }
    }
  }
  return CUBFF_OK;
}

}  // extern "C"
