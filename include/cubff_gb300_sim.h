// cubff_gb300_sim.h — C++ simulation API of the GB300 engine, with the names,
// fields and semantics of the reference's plugin API (common.h:55-139):
// SimulationParams, SimulationState, LanguageInterface and GetLanguage.
//
// The implementation (cubff_gb300/csrc/host/) runs the epoch loop of
// RunSimulation (common_language.h:345-596) on the device through the C ABI
// of include/cubff_gb300.h, and computes the callback statistics on the host.
// Differences from the reference: errors raise cubff::Error instead of
// calling exit(1); an unknown language name makes GetLanguage throw.
#ifndef CUBFF_GB300_SIM_H_
#define CUBFF_GB300_SIM_H_

#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

constexpr int kSingleTapeSize = 64;
constexpr int kSelfrepThreshold = 5;

inline constexpr const char *ResetColors() { return "\x1b[0;38:5:35;48:5:232m"; }

// common.h:58-72.
struct SimulationParams {
  size_t num_programs = 128 * 1024;
  size_t seed = 0;
  uint32_t mutation_prob = 1 << 18;  // out of 1 << 30
  std::optional<size_t> reset_interval = std::nullopt;
  std::optional<std::string> load_from = std::nullopt;
  std::optional<std::string> save_to = std::nullopt;
  size_t callback_interval = 128;
  size_t save_interval = 0;
  bool permute_programs = true;
  bool fixed_shuffle = false;
  bool zero_init = false;
  bool eval_selfrep = false;
  std::vector<std::vector<uint32_t>> allowed_interactions;
};

// common.h:74-91.
struct SimulationState {
  std::vector<uint8_t> soup;
  std::vector<uint32_t> shuffle_idx;
  std::array<std::array<uint8_t, 3>, 256> byte_colors;
  float elapsed_s;
  size_t total_ops;
  float mops_s;
  size_t epoch;
  float ops_per_run;
  size_t brotli_size;
  float brotli_bpb;
  float bytes_per_prog;
  float h0;
  float higher_entropy;
  std::array<std::pair<std::string, float>, 16> frequent_bytes;
  std::array<std::pair<std::string, float>, 16> uncommon_bytes;
  std::vector<size_t> replication_per_prog;
};

// common.h:93-111.
struct LanguageInterface {
  virtual void RunSingleProgram(std::string program, size_t stepcount, bool debug) const = 0;
  virtual void RunSingleParsedProgram(const std::vector<uint8_t> &parsed, size_t stepcount,
                                      bool debug) const = 0;
  virtual void PrintProgram(size_t pc_pos, const uint8_t *mem, size_t len,
                            const size_t *separators, size_t num_separators) const = 0;
  virtual void RunSimulation(const SimulationParams &params,
                             std::optional<std::string> initial_program,
                             std::function<bool(const SimulationState &)> callback) const = 0;
  virtual ~LanguageInterface() {}
  virtual size_t EvalSelfrep(std::string program, size_t epoch, size_t seed, bool debug) = 0;
  virtual size_t EvalParsedSelfrep(std::vector<uint8_t> &parsed, size_t epoch, size_t seed,
                                   bool debug) = 0;
  virtual std::vector<uint8_t> Parse(const std::string &program) = 0;
};

// The registry of the 13 languages (common.cc:22-40).  Throws cubff::Error
// for an unknown name.
const LanguageInterface *GetLanguage(const std::string &language);
std::vector<std::string> LanguageNames();

namespace cubff {

struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string &msg) : std::runtime_error(msg), status(st) {}
};

// The per-language host parts of the plugins (parse, display, colours).
std::vector<uint8_t> ParseProgram(int lang, const std::string &program);
std::string MapChar(int lang, uint8_t c);
void InitByteColors(int lang, std::array<std::array<uint8_t, 3>, 256> &byte_colors);
void PrintProgram(int lang, size_t pc_pos, const uint8_t *mem, size_t len,
                  const size_t *separators, size_t num_separators);

// Brotli size of a buffer with the reference's settings (quality 2, lgwin 24,
// generic mode; common_language.h:504-507), through the installed
// libbrotlienc loaded at run time.  Returns false when it is not installed.
bool BrotliSize(const uint8_t *data, size_t size, size_t *out);

}  // namespace cubff

#endif  // CUBFF_GB300_SIM_H_
