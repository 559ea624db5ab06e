// internal.h — host-side helpers shared by the engine's translation units.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/cubff_gb300.h"

namespace cubff {

// Records the calling thread's last error message; returns status.
int set_error(int status, const char *fmt, ...);
void clear_error();

#define CUBFF_CUDA_TRY(expr)                                                 \
  do {                                                                       \
    cudaError_t err_ = (expr);                                               \
    if (err_ != cudaSuccess)                                                 \
      return ::cubff::set_error(CUBFF_EDEVICE, "%s: %s (%s:%d)", #expr,      \
                                cudaGetErrorString(err_), __FILE__, __LINE__); \
  } while (0)

#define CUBFF_TRY(expr)           \
  do {                            \
    int st_ = (expr);             \
    if (st_ != CUBFF_OK) return st_; \
  } while (0)

// Launch arguments of one epoch of one soup (MutateAndRunPrograms).
struct EpochArgs {
  uint8_t *soup;
  const uint32_t *perm;                 // shuffle_idx of this epoch
  uint64_t n;                           // num_programs
  uint64_t num_indices;                 // pairs evaluated (k < num_indices)
  const uint64_t *d_num_indices;        // if set, overrides num_indices
  uint64_t epoch_key;                   // seed(epoch)
  uint32_t mutation_prob;
  unsigned long long *ops;              // += epoch op count
  unsigned long long *raw;              // += raw iterations (nullable)
};

// Launch arguments of a pipelined run of epochs [e0, e0 + n_epochs) of one
// soup (pipeline.cu).
struct PipeArgs {
  uint8_t *soup;
  const uint32_t *perm;                 // [n_epochs][n] shuffle_idx
  uint64_t n;
  uint64_t s0;                          // SplitMix64(params.seed)
  uint64_t e0;
  uint32_t n_epochs;
  uint32_t mutation_prob;
  const uint64_t *d_num_indices;        // [n_epochs] or nullptr (= n / 2)
  const uint4 *mutmask;                 // [n_epochs][n / 2] mutation masks
  const uint32_t *inv;                  // [n_epochs][n] position of program p in perm
  uint32_t *readycnt;                   // [n_epochs][n / 2] inputs published, zeroed
  uint32_t *queue;                      // [(n_epochs - 1) * n / 2] ready tasks + 1, zeroed
  uint32_t *qctl;                       // [0] head, [1] tail; zeroed
  int *error;                           // set when a bounded wait gives up
  unsigned long long *ops;              // [n_epochs][kCountSlots][2]: ops, raw
  uint32_t lanes_per_pair64;            // lanes per 64 pairs of an epoch (0 = default)
};
constexpr int kPipeCountSlots = 32;

// Launchers (epoch.cu / pairing.cu / pipeline.cu).
int launch_pipeline(int lang, const PipeArgs &a, int device, cudaStream_t stream);
int launch_mutation_masks(uint64_t s0, uint64_t e0, uint32_t n_epochs, uint64_t n, uint32_t prob,
                          uint4 *out, cudaStream_t stream);
int launch_inverse(const uint32_t *perm, uint32_t n_epochs, uint64_t n, uint32_t *inv,
                   cudaStream_t stream);
int launch_epoch(int lang, const EpochArgs &a, cudaStream_t stream);
int launch_init(uint64_t key, uint64_t n, uint8_t *soup, int zero_init,
                uint64_t count, cudaStream_t stream);
int launch_selfrep(int lang, const uint8_t *soup, uint64_t epoch_key,
                   uint64_t n, uint64_t count, uint64_t *result,
                   cudaStream_t stream);

size_t shuffle_scratch_bytes(uint64_t n, uint32_t n_epochs);
int launch_shuffle(uint64_t s0, uint64_t first_epoch, uint32_t n_epochs,
                   uint64_t n, uint32_t *out, void *scratch, cudaStream_t stream);
int launch_fixed(uint64_t first_epoch, uint32_t n_epochs, uint64_t n,
                 uint32_t *out, cudaStream_t stream);
int launch_cyclic(uint64_t first_epoch, uint32_t n_epochs, uint64_t n,
                  uint32_t *out, cudaStream_t stream);

}  // namespace cubff
