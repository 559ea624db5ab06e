// main.cc — command-line driver of the GB300 engine with the reference CLI's
// flags (main.cc:177-214) and its log format (main.cc:337-343, :391-401):
//
//   cubff_gb300/cubff_main --lang bff_noheads --max_epochs 256
//       --disable_output --log out.csv --seed 10248   (one command line)
//
// The soup runs on the device through LanguageInterface::RunSimulation.  The
// terminal UI prints a summary line per callback; PPM drawing is not provided.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <optional>
#include <string>
#include <vector>

#include "cubff_gb300_sim.h"

namespace {

struct Flags {
  std::map<std::string, std::string> values;
  std::map<std::string, bool> bools;
  std::optional<std::string> get(const std::string &k) const {
    auto it = values.find(k);
    if (it == values.end()) return std::nullopt;
    return it->second;
  }
  bool flag(const std::string &k, bool dflt) const {
    auto it = bools.find(k);
    return it == bools.end() ? dflt : it->second;
  }
};

const char *kBoolFlags[] = {"debug", "permute_programs", "fixed_shuffle", "zero_init",
                            "eval_selfrep", "disable_output"};
const char *kValueFlags[] = {"run", "run_steps", "num", "max_epochs", "seed", "mutation_prob",
                             "stopping_bpb", "initial_program", "log", "load", "checkpoint_dir",
                             "reset_interval", "lang", "interaction_pattern", "print_interval",
                             "save_interval", "clear_interval", "draw_to", "draw_to_2d",
                             "grid_width_2d", "stopping_selfrep_count"};

int usage() {
  fprintf(stderr, "usage: cubff_main --lang L [--num N] [--seed S] [--max_epochs E] "
                  "[--mutation_prob P] [--print_interval I] [--log FILE] [--load FILE] "
                  "[--checkpoint_dir DIR] [--save_interval I] [--reset_interval R] "
                  "[--interaction_pattern FILE] [--initial_program P] [--run P] "
                  "[--[no]permute_programs] [--[no]fixed_shuffle] [--[no]zero_init] "
                  "[--[no]eval_selfrep] [--[no]disable_output] ...\n");
  return 1;
}

bool parse(int argc, char **argv, Flags &f) {
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    if (a.rfind("--", 0) != 0) return false;
    a = a.substr(2);
    bool handled = false;
    for (const char *b : kBoolFlags) {
      if (a == b) f.bools[a] = true, handled = true;
      else if (a == std::string("no") + b) f.bools[b] = false, handled = true;
    }
    if (handled) continue;
    for (const char *v : kValueFlags) {
      if (a == v) {
        if (i + 1 >= argc) return false;
        f.values[a] = argv[++i];
        handled = true;
      }
    }
    if (!handled) {
      fprintf(stderr, "unknown flag --%s\n", a.c_str());
      return false;
    }
  }
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  Flags f;
  if (!parse(argc, argv, f) || !f.get("lang")) return usage();
  try {
    SimulationParams params;
    params.num_programs = std::stoull(f.get("num").value_or("131072"));
    params.seed = std::stoull(f.get("seed").value_or("0"));
    params.mutation_prob = static_cast<uint32_t>(
        std::round(std::stod(f.get("mutation_prob").value_or("0.000244140625")) * (1 << 30)));
    if (auto r = f.get("reset_interval")) params.reset_interval = std::stoull(*r);
    params.load_from = f.get("load");
    params.save_to = f.get("checkpoint_dir");
    params.save_interval = std::stoull(f.get("save_interval").value_or("256"));
    params.permute_programs = f.flag("permute_programs", true);
    params.fixed_shuffle = f.flag("fixed_shuffle", false);
    params.zero_init = f.flag("zero_init", false);
    params.eval_selfrep = f.flag("eval_selfrep", false);
    if (params.fixed_shuffle && (params.num_programs & (params.num_programs - 1)) != 0) {
      fprintf(stderr, "#programs must be a power of two for fixed shuffle\n");
      return 1;
    }
    const std::string pattern = f.get("interaction_pattern").value_or("");
    if (params.fixed_shuffle && !pattern.empty()) {
      fprintf(stderr, "fixed shuffle and interaction pattern are incompatible\n");
      return 1;
    }
    if (!pattern.empty()) {  // main.cc:281-299
      FILE *pf = fopen(pattern.c_str(), "r");
      if (!pf) {
        fprintf(stderr, "could not open interaction pattern file\n");
        return 1;
      }
      params.allowed_interactions.resize(params.num_programs);
      long long a, b;
      while (fscanf(pf, "%lld%lld", &a, &b) == 2) {
        if (static_cast<size_t>(a) >= params.num_programs ||
            static_cast<size_t>(b) >= params.num_programs) {
          fprintf(stderr, "invalid interaction pattern: programs not in [0, n) range.\n");
          fclose(pf);
          return 1;
        }
        params.allowed_interactions[a].push_back(static_cast<uint32_t>(b));
      }
      fclose(pf);
    }
    const size_t print_interval = std::stoull(f.get("print_interval").value_or("64"));
    const size_t clear_interval = std::stoull(f.get("clear_interval").value_or("2048"));
    std::optional<size_t> max_epochs, stopping_selfrep_count;
    std::optional<double> stopping_bpb;
    if (auto v = f.get("max_epochs")) max_epochs = std::stoull(*v);
    if (auto v = f.get("stopping_bpb")) stopping_bpb = std::stod(*v);
    if (auto v = f.get("stopping_selfrep_count")) stopping_selfrep_count = std::stoull(*v);
    if (stopping_selfrep_count && !params.eval_selfrep) {
      fprintf(stderr, "stopping_selfrep_count requires eval_selfrep\n");
      return 1;
    }
    if (print_interval == 0 || params.save_interval % print_interval != 0) {
      fprintf(stderr, "save interval must be divisible by print interval\n");
      return 1;
    }
    if (clear_interval % print_interval != 0) {
      fprintf(stderr, "clear interval must be divisible by print interval\n");
      return 1;
    }
    if (f.get("draw_to") || f.get("draw_to_2d"))
      fprintf(stderr, "note: frame drawing (--draw_to, --draw_to_2d) is not provided\n");
    params.callback_interval = print_interval;
    const LanguageInterface *language = GetLanguage(*f.get("lang"));
    if (auto run = f.get("run")) {
      printf("%s", ResetColors());
      const_cast<LanguageInterface *>(language)->RunSingleProgram(
          *run, std::stoull(f.get("run_steps").value_or("32768")), f.flag("debug", false));
      return 0;
    }
    FILE *logfile = nullptr;
    if (auto l = f.get("log")) {
      logfile = fopen(l->c_str(), "w");
      if (!logfile) {
        fprintf(stderr, "Could not open %s\n", l->c_str());
        return 1;
      }
      fprintf(logfile, params.eval_selfrep
                           ? "epoch,brotli_size,soup_size,higher_entropy,number_selfreps\n"
                           : "epoch,brotli_size,soup_size,higher_entropy\n");
    }
    const bool quiet = f.flag("disable_output", false);
    auto callback = [&](const SimulationState &st) {
      int repl = 0;
      for (size_t r : st.replication_per_prog) repl += r >= static_cast<size_t>(kSelfrepThreshold);
      if (!quiet) {
        printf("epoch %10zu  ops %14zu  MOps/s %12.3f  ops/run %8.3f  brotli %10zu  bpb %7.4f  "
               "H0 %7.4f  higher_entropy %9.6f%s\n",
               st.epoch, st.total_ops, st.mops_s, st.ops_per_run, st.brotli_size, st.brotli_bpb,
               st.h0, st.higher_entropy,
               params.eval_selfrep ? (" selfreps " + std::to_string(repl)).c_str() : "");
        fflush(stdout);
      }
      if (logfile) {
        if (params.eval_selfrep)
          fprintf(logfile, "%zu,%zu,%zu,%f,%d\n", st.epoch, st.brotli_size,
                  st.soup.size() / kSingleTapeSize, st.higher_entropy, repl);
        else
          fprintf(logfile, "%zu,%zu,%zu,%f\n", st.epoch, st.brotli_size,
                  st.soup.size() / kSingleTapeSize, st.higher_entropy);
        fflush(logfile);
      }
      if (max_epochs && st.epoch > *max_epochs) return true;  // main.cc:461
      if (stopping_bpb && st.brotli_bpb < *stopping_bpb) return true;
      if (stopping_selfrep_count && static_cast<size_t>(repl) >= *stopping_selfrep_count) return true;
      return false;
    };
    language->RunSimulation(params, f.get("initial_program"), callback);
    if (logfile) fclose(logfile);
  } catch (const std::exception &e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
