// server.cu — serving soup jobs (cubff_server_*): continuous admission by
// device-memory footprint and batched advancement of the running jobs.
//
// One worker thread per language, each with an engine of its own (its own
// streams and launch buffers, on the server's device), serves the jobs of
// that language.  Each round a worker
//   1. admits the queued jobs of its language in submission order while the
//      summed footprint of all running jobs stays within the budget (a job
//      of its language that does not fit is not skipped, so a large job
//      cannot starve behind smaller ones of the same language),
//   2. advances every job it runs by min(round_epochs, the epochs it has
//      left) in one run_soups call (pipelined launches shared by its running
//      jobs; a job near its end does not shorten the others' round),
//   3. retires the jobs that are done: soup bytes and op counts to the host,
//      device memory released.
// The workers run side by side, so a job that arrives while other
// languages' rounds are on the GPU starts at once, its launches overlapping
// theirs; within a language it joins at the next round.  A job's results
// equal cubff_soup_run's for the same parameters: run_soups gives every soup
// exactly its own epoch sequence.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "engine_impl.h"
#include "internal.h"

namespace {

struct Job {
  uint64_t id = 0;
  cubff_soup_params params{};
  uint64_t n_epochs = 0, done = 0, footprint = 0;
  cubff_soup *soup = nullptr;
  std::vector<uint64_t> ops;
  std::vector<uint8_t> result;  // final soup bytes
  int status = CUBFF_OK;
  double submit_s = 0, start_s = 0, finish_s = 0;
};

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The worker of one language.
struct LangWorker {
  int lang = 0;
  cubff_engine *eng = nullptr;                     // created by the worker
  std::vector<std::unique_ptr<Job>> running;       // worker only
  std::thread th;
};

}  // namespace

struct cubff_server {
  cubff_engine *eng = nullptr;  // the caller's engine: gives the device
  uint64_t budget = 0;
  uint32_t round_epochs = 64;
  std::chrono::steady_clock::time_point t0;

  std::mutex mu;
  std::condition_variable work_cv;  // workers wait for jobs or budget
  std::condition_variable done_cv;  // pollers wait for finished jobs
  bool stop = false;
  uint64_t next_id = 1;
  std::deque<std::unique_ptr<Job>> queued;           // guarded by mu
  uint64_t n_running = 0, running_bytes = 0;         // guarded by mu
  std::map<uint64_t, std::unique_ptr<Job>> finished; // guarded by mu
  std::deque<uint64_t> unreported;                   // finished ids not yet polled
  std::unique_ptr<LangWorker> workers[cubff::kNumLangs];  // created on a language's first job

  void loop(LangWorker *w);
  // True (mu held) when the first queued job of lang fits the budget.
  bool admissible(int lang) const;
  void admit(LangWorker *w);
  void retire(std::unique_ptr<Job> job, int status);
};

bool cubff_server::admissible(int lang) const {
  for (const auto &j : queued)
    if (j->params.lang == lang) return running_bytes + j->footprint <= budget;
  return false;
}

void cubff_server::admit(LangWorker *w) {
  std::vector<std::unique_ptr<Job>> take;
  {
    std::lock_guard<std::mutex> lk(mu);
    for (auto it = queued.begin(); it != queued.end();) {
      if ((*it)->params.lang != w->lang) {
        ++it;
        continue;
      }
      if (running_bytes + (*it)->footprint > budget) break;  // not skipped
      running_bytes += (*it)->footprint;
      take.push_back(std::move(*it));
      it = queued.erase(it);
    }
    n_running += take.size();
  }
  for (auto &job : take) {
    job->start_s = seconds_since(t0);
    int st = cubff_soup_create(w->eng, &job->params, &job->soup);
    if (st == CUBFF_OK) st = job->soup->ensure_buffers();
    if (st != CUBFF_OK) {
      retire(std::move(job), st);
      continue;
    }
    w->running.push_back(std::move(job));
  }
}

void cubff_server::retire(std::unique_ptr<Job> job, int status) {
  job->status = status;
  if (status == CUBFF_OK && job->soup) {
    job->result.resize(job->params.num_programs * cubff::kTape);
    job->status = cubff_soup_read(job->soup, job->result.data(), 0, job->result.size());
  }
  if (job->soup) cubff_soup_destroy(job->soup);
  job->soup = nullptr;
  job->finish_s = seconds_since(t0);
  {
    std::lock_guard<std::mutex> lk(mu);
    if (n_running) n_running--;
    running_bytes -= std::min(running_bytes, job->footprint);
    unreported.push_back(job->id);
    finished[job->id] = std::move(job);
  }
  done_cv.notify_all();
  work_cv.notify_all();  // budget freed: other workers may admit
}

void cubff_server::loop(LangWorker *w) {
  cudaSetDevice(eng->device);
  while (true) {
    {
      std::unique_lock<std::mutex> lk(mu);
      work_cv.wait(lk, [&] { return stop || !w->running.empty() || admissible(w->lang); });
      if (stop) break;
    }
    admit(w);
    if (w->running.empty()) continue;
    // Every job advances by its own quantum: round_epochs, or what it has
    // left (a job about to finish does not shorten the others' round).
    std::vector<cubff_soup *> soups;
    std::vector<uint64_t *> ops;
    std::vector<uint64_t> quantum;
    for (auto &j : w->running) {
      soups.push_back(j->soup);
      ops.push_back(j->ops.data() + j->done);
      quantum.push_back(std::min<uint64_t>(round_epochs, j->n_epochs - j->done));
    }
    const int st = cubff::run_soups(w->eng, soups.data(), static_cast<int>(soups.size()),
                                    round_epochs, ops.data(), nullptr, nullptr, quantum.data());
    std::vector<std::unique_ptr<Job>> keep;
    for (size_t q = 0; q < w->running.size(); q++) {
      auto &j = w->running[q];
      if (st != CUBFF_OK) {
        retire(std::move(j), st);
        continue;
      }
      j->done += quantum[q];
      if (j->done == j->n_epochs) retire(std::move(j), CUBFF_OK);
      else keep.push_back(std::move(j));
    }
    w->running.swap(keep);
  }
  for (auto &j : w->running)
    if (j->soup) cubff_soup_destroy(j->soup);
  w->running.clear();
}

using namespace cubff;

extern "C" {

int cubff_server_create(cubff_engine *engine, uint64_t hbm_budget_bytes, uint32_t round_epochs,
                        cubff_server **out) {
  if (!engine || !out || hbm_budget_bytes == 0)
    return set_error(CUBFF_EINVAL, "server_create: bad arguments");
  auto *s = new (std::nothrow) cubff_server();
  if (!s) return set_error(CUBFF_ENOMEM, "server_create: host allocation");
  s->eng = engine;
  s->budget = hbm_budget_bytes;
  s->round_epochs = round_epochs ? round_epochs : 64;
  s->t0 = std::chrono::steady_clock::now();
  *out = s;
  return CUBFF_OK;
}

int cubff_server_destroy(cubff_server *s) {
  if (!s) return CUBFF_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->work_cv.notify_all();
  for (auto &w : s->workers) {
    if (!w) continue;
    if (w->th.joinable()) w->th.join();
    if (w->eng) cubff_engine_destroy(w->eng);
  }
  delete s;
  return CUBFF_OK;
}

int cubff_server_submit(cubff_server *s, const cubff_soup_params *params, uint64_t n_epochs,
                        uint64_t *job_id) {
  if (!s || !params || n_epochs == 0) return set_error(CUBFF_EINVAL, "server_submit: bad arguments");
  const cubff_soup_params &p = *params;
  if (p.lang < 0 || p.lang >= kNumLangs)
    return set_error(CUBFF_ENOTFOUND, "server_submit: unknown language %d", p.lang);
  if (p.num_programs == 0 || p.num_programs % 2 != 0 || p.num_programs > (1ull << 31))
    return set_error(CUBFF_EINVAL, "server_submit: num_programs must be even, in (0, 2^31]");
  if (p.pairing < CUBFF_PAIR_SHUFFLE || p.pairing > CUBFF_PAIR_CYCLIC)
    return set_error(CUBFF_EINVAL, "server_submit: pairing %d is not served", p.pairing);
  if (p.pairing == CUBFF_PAIR_FIXED && (p.num_programs & (p.num_programs - 1)) != 0)
    return set_error(CUBFF_EINVAL, "server_submit: fixed shuffle needs a power-of-two size");
  auto job = std::make_unique<Job>();
  job->params = p;
  job->n_epochs = n_epochs;
  job->footprint = cubff_soup_footprint_bytes(&p);
  if (job->footprint > s->budget)
    return set_error(CUBFF_EINVAL, "server_submit: footprint %llu bytes over the budget %llu",
                     static_cast<unsigned long long>(job->footprint),
                     static_cast<unsigned long long>(s->budget));
  job->ops.assign(n_epochs, 0);
  job->submit_s = seconds_since(s->t0);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->workers[p.lang]) {
      auto w = std::make_unique<LangWorker>();
      w->lang = p.lang;
      int prev = 0;  // engine creation makes its device current: keep the caller's
      cudaGetDevice(&prev);
      const int st = cubff_engine_create(s->eng->device, &w->eng);
      cudaSetDevice(prev);
      if (st != CUBFF_OK) return st;
      LangWorker *wp = w.get();
      w->th = std::thread([s, wp] { s->loop(wp); });
      s->workers[p.lang] = std::move(w);
    }
    job->id = s->next_id++;
    if (job_id) *job_id = job->id;
    s->queued.push_back(std::move(job));
  }
  s->work_cv.notify_all();
  return CUBFF_OK;
}

int cubff_server_poll(cubff_server *s, cubff_job_info *out, int max_jobs, int *n_out,
                      double wait_s) {
  if (!s || !n_out || max_jobs < 0 || (max_jobs > 0 && !out))
    return set_error(CUBFF_EINVAL, "server_poll: bad arguments");
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->unreported.empty() && wait_s > 0)
    s->done_cv.wait_for(lk, std::chrono::duration<double>(wait_s),
                        [&] { return !s->unreported.empty(); });
  int n = 0;
  while (n < max_jobs && !s->unreported.empty()) {
    const uint64_t id = s->unreported.front();
    s->unreported.pop_front();
    auto it = s->finished.find(id);
    if (it == s->finished.end()) continue;
    const Job &j = *it->second;
    cubff_job_info &o = out[n++];
    o.job_id = j.id;
    o.status = j.status;
    o.num_programs = j.params.num_programs;
    o.n_epochs = j.n_epochs;
    o.total_ops = 0;
    for (uint64_t v : j.ops) o.total_ops += v;
    o.submit_s = j.submit_s;
    o.start_s = j.start_s;
    o.finish_s = j.finish_s;
  }
  *n_out = n;
  return CUBFF_OK;
}

int cubff_server_fetch(cubff_server *s, uint64_t job_id, uint8_t *soup_out, uint64_t *ops_out) {
  if (!s) return set_error(CUBFF_EINVAL, "server_fetch: null server");
  std::unique_ptr<Job> job;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->finished.find(job_id);
    if (it == s->finished.end())
      return set_error(CUBFF_ENOTFOUND, "server_fetch: job %llu is not finished or unknown",
                       static_cast<unsigned long long>(job_id));
    job = std::move(it->second);
    s->finished.erase(it);
  }
  if (soup_out && !job->result.empty())
    std::copy(job->result.begin(), job->result.end(), soup_out);
  if (ops_out) std::copy(job->ops.begin(), job->ops.end(), ops_out);
  return job->status;
}

int cubff_server_stats(cubff_server *s, uint64_t *queued, uint64_t *running, uint64_t *finished,
                       uint64_t *hbm_bytes) {
  if (!s) return set_error(CUBFF_EINVAL, "server_stats: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = s->queued.size();
  if (running) *running = s->n_running;
  if (finished) *finished = s->finished.size();
  if (hbm_bytes) *hbm_bytes = s->running_bytes;
  return CUBFF_OK;
}

}  // extern "C"
