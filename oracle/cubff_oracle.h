/* cubff_oracle.h — CPU oracle for the cubff epoch step (mutate -> pair -> run
 * -> split).  TEST INFRASTRUCTURE ONLY: tests, the smoke check and the CPU
 * baseline leg of the benchmark call it to compare against.  The product (the
 * cubff_gb300 package) never links or calls it.
 *
 * Every function restates the reference algorithm from its semantics; each
 * cites the reference file:line it follows (paths inside the cubff project).
 * Parity of this oracle with the reference CPU build is pinned by
 * tests/test_oracle_pins.py (the testdata brotli goldens and per-epoch
 * op/sha fixtures generated from the reference build).
 */
#ifndef CUBFF_ORACLE_H_
#define CUBFF_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Language ids: the 13 registered languages of the reference (one per *.cu
 * file, names from each file's name()).  The same order is used by the GPU
 * engine's language table. */
enum {
  ORC_BFF = 0,              /* bff.cu              */
  ORC_BFF_NOHEADS,          /* bff_noheads.cu      */
  ORC_BFF_NOHEADS_4BIT,     /* bff_noheads_4bit.cu */
  ORC_BFF_PERM,             /* bff_perm.cu         */
  ORC_BFF8,                 /* bff8.cu             */
  ORC_BFF8_NOHEADS,         /* bff8_noheads.cu     */
  ORC_BFF_SELFMOVE,         /* bff_selfmove.cu     */
  ORC_FORTH,                /* forth.cu            */
  ORC_FORTHCOPY,            /* forthcopy.cu        */
  ORC_FORTHTRIVIAL,         /* forthtrivial.cu     */
  ORC_FORTHTRIVIAL_RESET,   /* forthtrivial_reset.cu */
  ORC_SUBLEQ,               /* subleq.cu           */
  ORC_RSUBLEQ4,             /* rsubleq4.cu         */
  ORC_NUM_LANGS
};

/* Pairing modes of RunSimulation (common_language.h:433-486). */
enum {
  ORC_PAIR_SHUFFLE = 0,     /* permute_programs, Fisher-Yates           */
  ORC_PAIR_FIXED = 1,       /* permute_programs && fixed_shuffle        */
  ORC_PAIR_CYCLIC = 2,      /* !permute_programs                        */
  ORC_PAIR_PATTERN = 3      /* allowed_interactions non-empty           */
};

const char *oracle_language_name(int lang);
int oracle_language_id(const char *name);

uint64_t oracle_splitmix64(uint64_t x);
uint64_t oracle_seed(uint64_t params_seed, uint64_t x);

/* InitPrograms (common_language.h:138-155) for programs [0, count). */
void oracle_init_programs(uint64_t key, uint64_t num_programs, uint8_t *soup,
                          int zero_init, uint64_t count);

/* Pairings; each writes s[0..n) and returns num_indices. */
uint64_t oracle_pairing_shuffle(uint64_t params_seed, uint64_t epoch,
                                uint64_t n, uint32_t *s);
uint64_t oracle_pairing_fixed(uint64_t epoch, uint64_t n, uint32_t *s);
uint64_t oracle_pairing_cyclic(uint64_t epoch, uint64_t n, uint32_t *s);
/* Interaction lists in CSR form: program i may pair with
 * tgts[offs[i] .. offs[i+1]).  offs has n+1 entries. */
uint64_t oracle_pairing_pattern(uint64_t params_seed, uint64_t epoch,
                                uint64_t n, const uint32_t *offs,
                                const uint32_t *tgts, uint32_t *s);

/* Language::Evaluate on one 128-byte pair tape.  Returns the
 * reference-counted ops; *raw_steps (nullable) gets the loop iterations. */
uint64_t oracle_evaluate(int lang, uint8_t *tape, uint64_t stepcount,
                         uint64_t *raw_steps);

/* MutateAndRunPrograms (common_language.h:157-193) over all pairs of one
 * epoch.  epoch_key = seed(epoch).  Returns the op count of the epoch;
 * *raw_steps (nullable) gets the summed loop iterations. */
uint64_t oracle_mutate_and_run(int lang, uint8_t *soup, const uint32_t *s,
                               uint64_t epoch_key, uint32_t mutation_prob,
                               uint64_t num_programs, uint64_t num_indices,
                               int nthreads, uint64_t *raw_steps);

typedef struct {
  int lang;
  uint64_t num_programs;
  uint64_t seed;
  uint32_t mutation_prob;
  int pairing;                /* ORC_PAIR_* */
  const uint32_t *pat_offs;   /* ORC_PAIR_PATTERN only */
  const uint32_t *pat_tgts;
  uint64_t reset_interval;    /* 0 = never */
  int zero_init;
  int nthreads;               /* 0 = OpenMP default */
} oracle_sim;

/* Runs epochs [first_epoch, first_epoch + n_epochs) of the RunSimulation loop
 * (common_language.h:432-596) on soup, including resets.  ops_per_epoch and
 * raw_per_epoch are nullable arrays of n_epochs entries.  Returns 0 on
 * success, -1 on invalid arguments. */
int oracle_run_epochs(const oracle_sim *p, uint8_t *soup, uint64_t first_epoch,
                      uint64_t n_epochs, uint64_t *reset_index,
                      uint64_t *ops_per_epoch, uint64_t *raw_per_epoch);

/* CheckSelfRep (common_language.h:203-277) for programs [0, count):
 * result[i] = self-replication score of program i. */
void oracle_check_selfrep(int lang, const uint8_t *soup, uint64_t epoch_key,
                          uint64_t num_programs, uint64_t count,
                          uint64_t *result, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
