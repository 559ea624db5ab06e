// simulation.cc — LanguageInterface of the GB300 engine: the callback loop of
// Simulation<L>::RunSimulation (common_language.h:345-596) over the C ABI,
// the registry of the 13 languages, and the single-program helpers.
#include <dlfcn.h>
#include <errno.h>
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>

#include "cubff_gb300.h"
#include "cubff_gb300_sim.h"

namespace cubff {
namespace {

uint64_t splitmix64(uint64_t x) {  // common_language.h:131-136
  uint64_t z = x + 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

void check(int st) {
  if (st != CUBFF_OK) throw Error(st, cubff_last_error());
}

// One engine per process on the current device (CUBFF_DEVICE overrides).
cubff_engine *engine() {
  static std::mutex mu;
  static cubff_engine *eng = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!eng) {
    const char *d = std::getenv("CUBFF_DEVICE");
    check(cubff_engine_create(d ? std::atoi(d) : 0, &eng));
  }
  return eng;
}

struct SoupHandle {
  cubff_soup *h = nullptr;
  ~SoupHandle() {
    if (h) cubff_soup_destroy(h);
  }
};

typedef size_t (*MaxSizeFn)(size_t);
typedef int (*CompressFn)(int, int, int, size_t, const uint8_t *, size_t *, uint8_t *);

}  // namespace

bool BrotliSize(const uint8_t *data, size_t size, size_t *out) {
  static std::once_flag once;
  static MaxSizeFn max_size = nullptr;
  static CompressFn compress = nullptr;
  std::call_once(once, [] {
    void *h = dlopen("libbrotlienc.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libbrotlienc.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    max_size = reinterpret_cast<MaxSizeFn>(dlsym(h, "BrotliEncoderMaxCompressedSize"));
    compress = reinterpret_cast<CompressFn>(dlsym(h, "BrotliEncoderCompress"));
  });
  if (!max_size || !compress) return false;
  std::vector<uint8_t> buf(max_size(size));
  size_t sz = buf.size();
  if (!compress(2, 24, 0 /* BROTLI_MODE_GENERIC */, size, data, &sz, buf.data())) return false;
  *out = sz;
  return true;
}

namespace {

class Simulation : public LanguageInterface {
 public:
  explicit Simulation(int lang) : lang_(lang) {}

  std::vector<uint8_t> Parse(const std::string &program) override {
    return ParseProgram(lang_, program);
  }

  void PrintProgram(size_t pc_pos, const uint8_t *mem, size_t len, const size_t *separators,
                    size_t num_separators) const override {
    cubff::PrintProgram(lang_, pc_pos, mem, len, separators, num_separators);
  }

  // RunSingleParsedProgram (common_language.h:280-296): the pair tape is run
  // on the device by the epoch kernel's interpreter, whose step limit is 8192;
  // per-step debug printing is not provided.
  void RunSingleParsedProgram(const std::vector<uint8_t> &parsed, size_t stepcount,
                              bool debug) const override {
    uint8_t tape[2 * kSingleTapeSize] = {};
    std::memcpy(tape, parsed.data(), std::min(parsed.size(), sizeof(tape)));
    PrintProgram(2 * kSingleTapeSize, tape, 2 * kSingleTapeSize, nullptr, 0);
    if (stepcount != 8192 || debug)
      fprintf(stderr, "note: runs with the 8192-step limit of the epoch kernel, without step "
                      "printing\n");
    uint64_t ops = 0;
    check(cubff_eval_pair(lang_, tape, &ops, nullptr));
    printf("%s", ResetColors());
    printf("ops: %d\n\n", static_cast<int>(ops));
    PrintProgram(2 * kSingleTapeSize, tape, 2 * kSingleTapeSize, nullptr, 0);
  }

  void RunSingleProgram(std::string program, size_t stepcount, bool debug) const override {
    RunSingleParsedProgram(ParseProgram(lang_, program), stepcount, debug);
  }

  // EvalParsedSelfrep (common_language.h:326-342).  The device evaluation
  // prints no intermediate programs, so debug has no effect.
  size_t EvalParsedSelfrep(std::vector<uint8_t> &parsed, size_t epoch, size_t seed,
                           bool /*debug*/) override {
    uint8_t prog[kSingleTapeSize] = {};
    std::memcpy(prog, parsed.data(), std::min(parsed.size(), sizeof(prog)));
    const uint64_t key = splitmix64(splitmix64(seed) ^ splitmix64(epoch));
    uint64_t res = 0;
    check(cubff_eval_selfrep(lang_, prog, key, &res));
    return res;
  }

  size_t EvalSelfrep(std::string program, size_t epoch, size_t seed, bool debug) override {
    std::vector<uint8_t> parsed = ParseProgram(lang_, program);
    return EvalParsedSelfrep(parsed, epoch, seed, debug);
  }

  void RunSimulation(const SimulationParams &params, std::optional<std::string> initial_program,
                     std::function<bool(const SimulationState &)> callback) const override;

 private:
  int lang_;
};

// Callback statistics of common_language.h:504-561; counts = the soup's byte
// histogram (counted on the device).
void fill_stats(int lang, SimulationState &st, size_t num_programs, size_t insn, size_t num_runs,
                const uint64_t *counts) {
  size_t bsize = 0;
  static bool warned = false;
  if (!BrotliSize(st.soup.data(), st.soup.size(), &bsize) && !warned) {
    fprintf(stderr, "cubff: libbrotlienc not found; brotli_size is reported as 0\n");
    warned = true;
  }
  std::vector<uint8_t> sorted(256);
  double h0 = 0;
  for (size_t i = 0; i < 256; i++) {
    sorted[i] = static_cast<uint8_t>(i);
    const double frac = counts[i] * 1.0 / st.soup.size();
    h0 -= counts[i] ? frac * std::log2(frac) : 0.0;
  }
  // Most frequent first; ties by the larger byte value first (:531-533).
  std::sort(sorted.begin(), sorted.end(), [&](uint8_t a, uint8_t b) {
    return std::make_pair(counts[b], b) < std::make_pair(counts[a], a);
  });
  const double bpb = bsize * 8.0 / (num_programs * kSingleTapeSize);
  st.ops_per_run = num_runs ? insn * 1.0 / num_runs : 0.0f;
  st.brotli_size = bsize;
  st.brotli_bpb = bpb;
  st.bytes_per_prog = bsize * 1.0 / num_programs;
  st.h0 = h0;
  st.higher_entropy = h0 - bpb;
  for (size_t i = 0; i < st.frequent_bytes.size(); i++) {
    const uint8_t c = sorted[i];
    st.frequent_bytes[i] = {MapChar(lang, c), counts[c] * 1.0f / st.soup.size()};
  }
  for (size_t i = 0; i < st.uncommon_bytes.size(); i++) {
    const uint8_t c = sorted[256 - st.uncommon_bytes.size() + i];
    st.uncommon_bytes[i] = {MapChar(lang, c), counts[c] * 1.0f / st.soup.size()};
  }
}

void Simulation::RunSimulation(const SimulationParams &params,
                               std::optional<std::string> initial_program,
                               std::function<bool(const SimulationState &)> callback) const {
  using clock = std::chrono::high_resolution_clock;
  size_t num_programs = params.num_programs;
  uint64_t reset_index = 1, epoch = 0;
  std::vector<uint8_t> loaded;
  if (params.load_from) {  // common_language.h:354-360, :398-403
    FILE *f = fopen(params.load_from->c_str(), "rb");
    if (!f) throw Error(CUBFF_EINVAL, "Could not open " + *params.load_from + ": " + strerror(errno));
    uint64_t hdr[3];
    const bool ok = fread(hdr, sizeof(uint64_t), 3, f) == 3;
    if (ok) {
      reset_index = hdr[0];
      num_programs = hdr[1];
      epoch = hdr[2];
      loaded.resize(num_programs * kSingleTapeSize);
    }
    const bool ok2 = ok && fread(loaded.data(), 1, loaded.size(), f) == loaded.size();
    fclose(f);
    if (!ok2) throw Error(CUBFF_EINVAL, "truncated checkpoint " + *params.load_from);
  }
  if (num_programs % 2 != 0) throw Error(CUBFF_EINVAL, "num_programs % 2 == 0 is false");
  if (params.callback_interval == 0) throw Error(CUBFF_EINVAL, "callback_interval must be > 0");

  cubff_soup_params sp{};
  sp.lang = lang_;
  sp.num_programs = num_programs;
  sp.seed = params.seed;
  sp.mutation_prob = params.mutation_prob;
  sp.pairing = !params.allowed_interactions.empty()
                   ? CUBFF_PAIR_PATTERN
                   : (params.permute_programs ? (params.fixed_shuffle ? CUBFF_PAIR_FIXED
                                                                      : CUBFF_PAIR_SHUFFLE)
                                              : CUBFF_PAIR_CYCLIC);
  sp.reset_interval = params.reset_interval.value_or(0);
  sp.zero_init = params.zero_init;
  SoupHandle soup;
  check(cubff_soup_create(engine(), &sp, &soup.h));  // init with seed(0), :371-373
  if (sp.pairing == CUBFF_PAIR_PATTERN) {
    std::vector<uint32_t> offs(num_programs + 1, 0), tgts;
    for (size_t i = 0; i < num_programs; i++) {
      if (i < params.allowed_interactions.size())
        tgts.insert(tgts.end(), params.allowed_interactions[i].begin(),
                    params.allowed_interactions[i].end());
      offs[i + 1] = static_cast<uint32_t>(tgts.size());
    }
    check(cubff_soup_set_pattern(soup.h, offs.data(), tgts.data()));
  }
  if (initial_program) {  // :375-378
    std::vector<uint8_t> parsed = ParseProgram(lang_, *initial_program);
    const size_t nb = std::min(parsed.size(), num_programs * kSingleTapeSize);
    check(cubff_soup_write(soup.h, parsed.data(), 0, nb));
  }
  if (params.save_to) {
    if (mkdir(params.save_to->c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH) == -1 && errno != EEXIST)
      throw Error(CUBFF_EINVAL, "could not create " + *params.save_to);
  }
  if (params.load_from) {
    check(cubff_soup_set_epoch(soup.h, epoch, reset_index));
    check(cubff_soup_write(soup.h, loaded.data(), 0, loaded.size()));
  }

  SimulationState state;
  state.soup.resize(num_programs * kSingleTapeSize);
  state.replication_per_prog.assign(num_programs, 0);
  state.shuffle_idx.resize(num_programs);
  InitByteColors(lang_, state.byte_colors);

  size_t total_ops = 0;
  const auto sim_start = clock::now();
  auto start = sim_start;
  const uint64_t ci = params.callback_interval;

  // One segment of the loop: the epochs up to and including the next
  // callback epoch (e % callback_interval == 0).
  struct Segment {
    uint64_t cb_epoch = 0, k = 0;
    std::vector<uint64_t> ops, ni;
    std::vector<uint32_t> shuffle;
    int status = CUBFF_OK;
    std::string error;
  };
  auto run_segment = [&](Segment &g) {
    uint64_t e0 = 0, ri = 0;
    g.status = cubff_soup_get_epoch(soup.h, &e0, &ri);
    if (g.status == CUBFF_OK) {
      g.cb_epoch = e0 + (ci - e0 % ci) % ci;
      g.k = g.cb_epoch - e0 + 1;
      g.ops.assign(g.k, 0);
      g.ni.assign(g.k, 0);
      g.shuffle.resize(num_programs);
      g.status = cubff_soup_run(soup.h, g.k, g.ops.data(), nullptr, g.shuffle.data(), g.ni.data());
    }
    if (g.status != CUBFF_OK) g.error = cubff_last_error();
  };
  // While the host computes a callback's statistics (brotli) and runs the
  // callback, the next segment already runs on the device, from a worker
  // thread.  The callback sees the soup as it was at its epoch (copied to
  // the host before the next segment starts); if it stops the run, the extra
  // segment's work is dropped with the soup.
  Segment cur, next;
  struct Joiner {  // declared after the segments, so it joins before they go
    std::thread t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } ahead;
  run_segment(cur);
  while (true) {
    if (cur.status != CUBFF_OK) throw Error(cur.status, cur.error);
    const auto stop = clock::now();
    size_t insn = 0, num_runs = 0;
    for (uint64_t q = 0; q < cur.k; q++) {
      insn += cur.ops[q];
      num_runs += cur.ni[q];
    }
    total_ops += insn;
    uint64_t e_now = 0, ri = 0;
    check(cubff_soup_get_epoch(soup.h, &e_now, &ri));
    check(cubff_soup_read(soup.h, state.soup.data(), 0, state.soup.size()));
    uint64_t counts[256];
    check(cubff_soup_histogram(soup.h, counts));
    state.shuffle_idx.assign(cur.shuffle.begin(), cur.shuffle.end());
    if (params.eval_selfrep) {  // :563-569, on the soup of this callback's epoch
      std::vector<uint64_t> rep(num_programs);
      check(cubff_soup_selfrep(soup.h, cur.cb_epoch, rep.data()));
      for (size_t i = 0; i < num_programs; i++) state.replication_per_prog[i] = rep[i];
    }
    next = Segment();
    ahead.t = std::thread([&] { run_segment(next); });
    const float elapsed = std::chrono::duration_cast<std::chrono::microseconds>(stop - start).count() * 1e-6;
    const float sim_elapsed =
        std::chrono::duration_cast<std::chrono::microseconds>(stop - sim_start).count() * 1e-6;
    fill_stats(lang_, state, num_programs, insn, num_runs, counts);
    state.elapsed_s = sim_elapsed;
    state.total_ops = total_ops;
    state.mops_s = elapsed > 0 ? insn * 1.0 / elapsed * 1e-6 : 0.0f;
    state.epoch = cur.cb_epoch + 1;
    if (params.save_to && params.save_interval && cur.cb_epoch % params.save_interval == 0) {
      char path[4096];  // :570-581
      snprintf(path, sizeof(path), "%s/%010llu.dat", params.save_to->c_str(),
               static_cast<unsigned long long>(cur.cb_epoch));
      FILE *f = fopen(path, "wb");
      if (!f) throw Error(CUBFF_EINVAL, std::string("Could not open ") + path);
      const uint64_t hdr[3] = {ri, num_programs, cur.cb_epoch + 1};
      fwrite(hdr, sizeof(uint64_t), 3, f);
      fwrite(state.soup.data(), 1, state.soup.size(), f);
      fclose(f);
    }
    const bool done = callback(state);
    ahead.t.join();
    if (done) break;
    start = stop;
    cur = std::move(next);
  }
}

struct Registry {
  std::vector<std::unique_ptr<Simulation>> langs;
  Registry() {
    for (int i = 0; i < cubff_language_count(); i++) langs.emplace_back(new Simulation(i));
  }
};

Registry &registry() {
  static Registry r;
  return r;
}

}  // namespace
}  // namespace cubff

const LanguageInterface *GetLanguage(const std::string &language) {
  const int id = cubff_language_id(language.c_str());
  if (id < 0) {
    std::string msg = "Unknown language `" + language + "`\nAvailable languages:\n";
    for (const auto &n : LanguageNames()) msg += n + "\n";
    throw cubff::Error(CUBFF_ENOTFOUND, msg);
  }
  return cubff::registry().langs[id].get();
}

std::vector<std::string> LanguageNames() {
  std::vector<std::string> out;
  for (int i = 0; i < cubff_language_count(); i++) out.emplace_back(cubff_language_name(i));
  return out;
}
