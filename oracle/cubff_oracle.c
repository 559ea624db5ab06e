/* cubff_oracle.c — CPU oracle for the cubff epoch step.
 *
 * TEST INFRASTRUCTURE ONLY (see cubff_oracle.h).  A plain-C restatement of the
 * reference's CPU semantics, written from the reference's behaviour; every
 * function cites the reference file:line it follows.  Pinned against the
 * reference CPU build by tests/test_oracle_pins.py.
 */
#include "cubff_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TAPE 64          /* kSingleTapeSize, common.h:55 */
#define PAIR (2 * TAPE)  /* pair tape */
#define STEP_LIMIT 8192  /* common_language.h:184 */

/* ------------------------------------------------------------------------ */
/* RNG: SplitMix64 finaliser (common_language.h:131-136), public algorithm
 * (Steele, Lea, Flood 2014), and the seed() lambda (common_language.h:367). */

uint64_t oracle_splitmix64(uint64_t x) {
  uint64_t z = x + 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

uint64_t oracle_seed(uint64_t params_seed, uint64_t x) {
  return oracle_splitmix64(oracle_splitmix64(params_seed) ^
                           oracle_splitmix64(x));
}

/* ------------------------------------------------------------------------ */
/* Language tables. */

static const char *const kNames[ORC_NUM_LANGS] = {
    "bff",          "bff_noheads",  "bff_noheads_4bit", "bff_perm",
    "bff8",         "bff8_noheads", "bff_selfmove",     "forth",
    "forthcopy",    "forthtrivial", "forthtrivial_reset", "subleq",
    "rsubleq4"};

const char *oracle_language_name(int lang) {
  return (lang >= 0 && lang < ORC_NUM_LANGS) ? kNames[lang] : NULL;
}

int oracle_language_id(const char *name) {
  for (int i = 0; i < ORC_NUM_LANGS; i++)
    if (strcmp(kNames[i], name) == 0) return i;
  return -1;
}

/* BFF op kinds (bff.inc.h:26-39). */
enum { B_LS, B_LE, B_PLUS, B_MINUS, B_C01, B_C10, B_DEC0, B_INC0, B_DEC1,
       B_INC1, B_NULL, B_NOOP };
/* BFF step logic: default scanning loops (bff.inc.h:289-349), bff8's
 * jump-by-8 loops (bff8.cu:23-65), bff_selfmove's (bff_selfmove.cu:55-98). */
enum { LOGIC_SCAN, LOGIC_JUMP8, LOGIC_SELFMOVE };

/* Forth op kinds (forth.inc.h:26-48). */
enum { F_WRITE0, F_WRITE1, F_WRITE, F_READ, F_READ0, F_READ1, F_DUP, F_DROP,
       F_SWAP, F_IF0, F_INC, F_DEC, F_ADD, F_SUB, F_COPY, F_COPY0, F_COPY1,
       F_XOR, F_CONST, F_JMP, F_NOOP };

static uint8_t bff_ops[7][256];
static uint8_t forth_ops[4][256];
static int tables_ready = 0;

static void build_tables(void) {
  if (tables_ready) return;
  /* Default BFF table (bff.inc.h:58-85). */
  uint8_t def[256];
  for (int c = 0; c < 256; c++) def[c] = B_NOOP;
  def['['] = B_LS; def[']'] = B_LE; def['+'] = B_PLUS; def['-'] = B_MINUS;
  def['.'] = B_C01; def[','] = B_C10; def['<'] = B_DEC0; def['>'] = B_INC0;
  def['{'] = B_DEC1; def['}'] = B_INC1; def[0] = B_NULL;
  memcpy(bff_ops[ORC_BFF], def, 256);
  memcpy(bff_ops[ORC_BFF_NOHEADS], def, 256);
  memcpy(bff_ops[ORC_BFF8], def, 256);
  memcpy(bff_ops[ORC_BFF8_NOHEADS], def, 256);
  /* bff_noheads_4bit.cu:22-49: op of the low nibble. */
  static const uint8_t nib[16] = {B_NULL, B_NOOP, B_NOOP, B_NOOP, B_NOOP,
                                  B_NOOP, B_LS,   B_LE,   B_PLUS, B_MINUS,
                                  B_C01,  B_C10,  B_DEC0, B_INC0, B_DEC1,
                                  B_INC1};
  for (int c = 0; c < 256; c++) bff_ops[ORC_BFF_NOHEADS_4BIT][c] = nib[c & 15];
  /* bff_perm.cu:23-50. */
  static const uint8_t perm[11] = {B_NULL, B_DEC0, B_INC0, B_DEC1, B_INC1,
                                   B_PLUS, B_MINUS, B_C01, B_C10, B_LS, B_LE};
  for (int c = 0; c < 256; c++)
    bff_ops[ORC_BFF_PERM][c] = c < 11 ? perm[c] : B_NOOP;
  /* bff_selfmove.cu:24-45. */
  static const uint8_t sm[7] = {B_INC0, B_DEC0, B_PLUS, B_MINUS, B_C10, B_LS,
                                B_LE};
  for (int c = 0; c < 256; c++)
    bff_ops[ORC_BFF_SELFMOVE][c] = c < 7 ? sm[c] : B_NOOP;

  /* Forth tables: forth.inc.h:53-85, forthcopy.cu:21-51,
   * forthtrivial.cu:21-55 (also used by forthtrivial_reset.cu:22-56). */
  for (int t = 0; t < 4; t++)
    for (int c = 0; c < 256; c++)
      forth_ops[t][c] = c >= 128 ? F_JMP : (c >= 64 ? F_CONST : F_NOOP);
  static const uint8_t f_def[12] = {F_READ0, F_READ1, F_WRITE0, F_WRITE1,
                                    F_DUP,   F_DROP,  F_SWAP,   F_IF0,
                                    F_INC,   F_DEC,   F_ADD,    F_SUB};
  static const uint8_t f_copy[12] = {F_READ, F_WRITE, F_COPY, F_XOR,
                                     F_DUP,  F_DROP,  F_SWAP, F_IF0,
                                     F_INC,  F_DEC,   F_ADD,  F_SUB};
  for (int c = 0; c < 12; c++) {
    forth_ops[0][c] = f_def[c];
    forth_ops[1][c] = f_copy[c];
    forth_ops[2][c] = f_def[c];
    forth_ops[3][c] = f_def[c];
  }
  forth_ops[2][0xC] = forth_ops[3][0xC] = F_COPY0;
  forth_ops[2][0xD] = forth_ops[3][0xD] = F_COPY1;
  __atomic_store_n(&tables_ready, 1, __ATOMIC_RELEASE);
}

/* ------------------------------------------------------------------------ */
/* BFF family: Evaluate (bff.inc.h:356-389) with InitialState
 * (bff.inc.h:269-283) and the per-variant EvaluateOne. */

static uint64_t bff_eval(const uint8_t *op, int heads, int logic, uint8_t *t,
                         uint64_t stepcount, uint64_t *raw) {
  int h0, h1, pc;
  if (heads) {
    h0 = t[0] % PAIR;
    h1 = t[1] % PAIR;
    pc = 2;
  } else {
    h0 = h1 = PAIR;
    pc = 0;
  }
  uint64_t i = 0, nskip = 0;
  for (; i < stepcount; i++) {
    h0 &= PAIR - 1;
    h1 &= PAIR - 1;
    int cmd = 1;
    switch (op[t[pc]]) {
      case B_DEC0: h0--; break;
      case B_INC0: h0++; break;
      case B_DEC1:
        if (logic == LOGIC_SELFMOVE) cmd = 0; else h1--;
        break;
      case B_INC1:
        if (logic == LOGIC_SELFMOVE) cmd = 0; else h1++;
        break;
      case B_PLUS: t[h0]++; break;
      case B_MINUS: t[h0]--; break;
      case B_C01:
        if (logic == LOGIC_SELFMOVE) cmd = 0; else t[h1] = t[h0];
        break;
      case B_C10:
        t[h0] = t[h1];
        if (logic == LOGIC_SELFMOVE) h1++;
        break;
      case B_LS: {
        int zero = logic == LOGIC_SCAN ? op[t[h0]] == B_NULL : t[h0] == 0;
        if (!zero) break;
        if (logic == LOGIC_JUMP8) {
          pc += 8;
          break;
        }
        /* forward scan for the matching ']' (bff.inc.h:318-329) */
        int depth = 1;
        pc++;
        for (; pc < PAIR && depth > 0; pc++) {
          if (op[t[pc]] == B_LE) depth--;
          if (op[t[pc]] == B_LS) depth++;
        }
        pc--;
        if (depth != 0) pc = PAIR;
        break;
      }
      case B_LE: {
        int zero = logic == LOGIC_SCAN ? op[t[h0]] == B_NULL : t[h0] == 0;
        if (zero) break;
        if (logic == LOGIC_JUMP8) {
          pc -= 8;
          break;
        }
        /* backward scan for the matching '[' (bff.inc.h:332-343) */
        int depth = 1;
        pc--;
        for (; pc >= 0 && depth > 0; pc--) {
          if (op[t[pc]] == B_LE) depth++;
          if (op[t[pc]] == B_LS) depth--;
        }
        pc++;
        if (depth != 0) pc = -1;
        break;
      }
      default:
        cmd = 0;
    }
    if (!cmd) nskip++;
    if (pc < 0) {
      i++;
      break;
    }
    pc++;
    if (pc >= PAIR) {
      i++;
      break;
    }
  }
  if (raw) *raw = i;
  return i - nskip;
}

/* ------------------------------------------------------------------------ */
/* Forth family: Stack (forth.inc.h:236-249), EvaluateOne (:250-373),
 * Evaluate (:379-397); forthtrivial_reset's Reset/ResetIf and its Write1 /
 * Copy0 (forthtrivial_reset.cu:58-72, :157-166, :215-223). */

typedef struct {
  uint8_t d[128];
  int sp;
  int overflow;
} fstack;

static inline void f_push(fstack *s, uint8_t v) {
  if (s->sp != 128) s->d[s->sp++] = v; else s->overflow = 1;
}
static inline uint8_t f_pop(fstack *s) {
  return s->sp == 0 ? 0 : s->d[--s->sp];
}

static void forth_reset(uint8_t *t, int pos) {
  uint64_t seed = 0;
  for (int i = 0; i < PAIR; i++) seed = oracle_splitmix64(seed ^ t[i]);
  for (int i = 0; i < TAPE; i++)
    t[i] = (uint8_t)oracle_splitmix64(seed * TAPE * TAPE +
                                      (uint64_t)(pos * TAPE) + (uint64_t)i);
}

static uint64_t forth_eval(const uint8_t *op, int with_reset, uint8_t *t,
                           uint64_t stepcount, uint64_t *raw) {
  fstack st;
  st.sp = 0;
  st.overflow = 0;
  int pos = 0;
  uint64_t i = 0, nops = 0;
  for (; i < stepcount; i++) {
    uint8_t c = t[pos];
    switch (op[c]) {
      case F_READ0: { int a = f_pop(&st) % TAPE; f_push(&st, t[a]); break; }
      case F_READ1: { int a = f_pop(&st) % TAPE; f_push(&st, t[TAPE + a]); break; }
      case F_READ: { int a = f_pop(&st) % PAIR; f_push(&st, t[a]); break; }
      case F_WRITE: {
        uint8_t v = f_pop(&st);
        int a = f_pop(&st) % PAIR;
        t[a] = v;
        break;
      }
      case F_WRITE0: {
        uint8_t v = f_pop(&st);
        int a = f_pop(&st) % TAPE;
        t[a] = v;
        break;
      }
      case F_WRITE1: {
        uint8_t v = f_pop(&st);
        int a = f_pop(&st) % TAPE;
        if (with_reset && t[TAPE + a] == 0x13) forth_reset(t, pos);
        else t[TAPE + a] = v;
        break;
      }
      case F_DUP: { uint8_t v = f_pop(&st); f_push(&st, v); f_push(&st, v); break; }
      case F_DROP: f_pop(&st); break;
      case F_SWAP: {
        uint8_t a = f_pop(&st), b = f_pop(&st);
        f_push(&st, a);
        f_push(&st, b);
        break;
      }
      case F_IF0: {
        uint8_t v = f_pop(&st);
        if (v) pos++;
        f_push(&st, v);
        break;
      }
      case F_INC: f_push(&st, (uint8_t)(f_pop(&st) + 1)); break;
      case F_DEC: f_push(&st, (uint8_t)(f_pop(&st) - 1)); break;
      case F_ADD: {
        uint8_t a = f_pop(&st), b = f_pop(&st);
        f_push(&st, (uint8_t)(a + b));
        break;
      }
      case F_SUB: {
        uint8_t a = f_pop(&st), b = f_pop(&st);
        f_push(&st, (uint8_t)(a - b));
        break;
      }
      case F_CONST: f_push(&st, c & 63); break;
      case F_COPY0: {
        int a = f_pop(&st) % TAPE;
        if (with_reset && t[TAPE + a] == 0x13) forth_reset(t, pos);
        else t[TAPE + a] = t[a];
        break;
      }
      case F_COPY1: { int a = f_pop(&st) % TAPE; t[a] = t[TAPE + a]; break; }
      case F_COPY: {
        int to = f_pop(&st) % PAIR;
        int from = f_pop(&st) % PAIR;
        t[to] = t[from];
        break;
      }
      case F_XOR: f_push(&st, f_pop(&st) ^ 64); break;
      case F_JMP: {
        int a = (c & 63) + 1;
        pos += (c & 64) ? -a : a;
        pos--;
        break;
      }
      default:
        nops++;
    }
    pos++;
    if (pos >= PAIR || pos < 0 || st.overflow) {
      i++;
      break;
    }
  }
  if (raw) *raw = i;
  return i - nops;
}

/* ------------------------------------------------------------------------ */
/* SUBLEQ (subleq.cu:109-133) and RSUBLEQ4 (rsubleq4.cu:116-141). */

static uint64_t subleq_eval(uint8_t *t, uint64_t stepcount, uint64_t *raw) {
  int pos = 0;
  uint64_t i = 0;
  for (; i < stepcount; i++) {
    int a = t[pos] % PAIR, b = t[pos + 1] % PAIR;
    t[a] -= t[b];
    if ((t[a] & 0x80) || t[a] == 0) pos = t[pos + 2];
    else pos += 3;
    if (pos + 3 > PAIR || pos < 0) {
      i++;
      break;
    }
  }
  if (raw) *raw = i;
  return i;
}

static uint64_t rsubleq4_eval(uint8_t *t, uint64_t stepcount, uint64_t *raw) {
  int pos = 0;
  uint64_t i = 0;
  for (; i < stepcount; i++) {
    int a = (pos + t[pos]) % PAIR;
    int b = (pos + t[pos + 1]) % PAIR;
    int c = (pos + t[pos + 2]) % PAIR;
    t[a] = (uint8_t)(t[b] - t[c]);
    if ((t[a] & 0x80) || t[a] == 0) pos += (int8_t)t[pos + 3];
    else pos += 4;
    if (pos + 4 > PAIR || pos < 0) {
      i++;
      break;
    }
  }
  if (raw) *raw = i;
  return i;
}

uint64_t oracle_evaluate(int lang, uint8_t *tape, uint64_t stepcount,
                         uint64_t *raw) {
  build_tables();
  switch (lang) {
    case ORC_BFF: return bff_eval(bff_ops[lang], 1, LOGIC_SCAN, tape, stepcount, raw);
    case ORC_BFF_NOHEADS: return bff_eval(bff_ops[lang], 0, LOGIC_SCAN, tape, stepcount, raw);
    case ORC_BFF_NOHEADS_4BIT: return bff_eval(bff_ops[lang], 0, LOGIC_SCAN, tape, stepcount, raw);
    case ORC_BFF_PERM: return bff_eval(bff_ops[lang], 1, LOGIC_SCAN, tape, stepcount, raw);
    case ORC_BFF8: return bff_eval(bff_ops[lang], 1, LOGIC_JUMP8, tape, stepcount, raw);
    case ORC_BFF8_NOHEADS: return bff_eval(bff_ops[lang], 0, LOGIC_JUMP8, tape, stepcount, raw);
    case ORC_BFF_SELFMOVE: return bff_eval(bff_ops[lang], 1, LOGIC_SELFMOVE, tape, stepcount, raw);
    case ORC_FORTH: return forth_eval(forth_ops[0], 0, tape, stepcount, raw);
    case ORC_FORTHCOPY: return forth_eval(forth_ops[1], 0, tape, stepcount, raw);
    case ORC_FORTHTRIVIAL: return forth_eval(forth_ops[2], 0, tape, stepcount, raw);
    case ORC_FORTHTRIVIAL_RESET: return forth_eval(forth_ops[3], 1, tape, stepcount, raw);
    case ORC_SUBLEQ: return subleq_eval(tape, stepcount, raw);
    case ORC_RSUBLEQ4: return rsubleq4_eval(tape, stepcount, raw);
  }
  if (raw) *raw = 0;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* InitPrograms (common_language.h:138-155). */

void oracle_init_programs(uint64_t key, uint64_t n, uint8_t *soup,
                          int zero_init, uint64_t count) {
#pragma omp parallel for schedule(static)
  for (uint64_t idx = 0; idx < count; idx++) {
    for (uint64_t i = 0; i < TAPE; i++)
      soup[idx * TAPE + i] =
          zero_init ? 0
                    : (uint8_t)oracle_splitmix64(TAPE * n * key + TAPE * idx + i);
  }
}

/* ------------------------------------------------------------------------ */
/* Pairings (common_language.h:418-486). */

/* do_shuffle (common_language.h:418-424): serial Fisher-Yates, keyed by
 * seed(epoch * len + i). */
static void fisher_yates(uint64_t params_seed, uint64_t epoch, uint32_t *b,
                         uint64_t len) {
  const uint64_t s0 = oracle_splitmix64(params_seed);
  for (uint64_t i = len; i-- > 0;) {
    uint64_t key = oracle_splitmix64(s0 ^ oracle_splitmix64(epoch * len + i));
    uint64_t j = oracle_splitmix64(key) % (i + 1);
    uint32_t tmp = b[i];
    b[i] = b[j];
    b[j] = tmp;
  }
}

uint64_t oracle_pairing_shuffle(uint64_t params_seed, uint64_t epoch,
                                uint64_t n, uint32_t *s) {
  for (uint64_t i = 0; i < n; i++) s[i] = (uint32_t)i;
  fisher_yates(params_seed, epoch, s, n);
  return n / 2;
}

/* common_language.h:468-474. */
uint64_t oracle_pairing_fixed(uint64_t epoch, uint64_t n, uint32_t *s) {
  uint64_t flip = epoch & 1;
  uint64_t max_pow2 = 31 - __builtin_clz((unsigned)n);
  uint64_t offset = (1ULL << (epoch % max_pow2 + 1)) - 1;
  for (uint64_t i = 0; i < n; i++) s[i] = (uint32_t)(((i * offset) % n) ^ flip);
  return n / 2;
}

/* common_language.h:478-486. */
uint64_t oracle_pairing_cyclic(uint64_t epoch, uint64_t n, uint32_t *s) {
  for (uint64_t i = 0; i < n; i++)
    s[i] = (epoch % 2 == 1) ? (uint32_t)i : (uint32_t)(i == 0 ? n - 1 : i - 1);
  return n / 2;
}

/* common_language.h:435-463: greedy matching in shuffled order, each program
 * proposing one neighbour drawn by seed(seed(epoch) ^ seed(i)). */
uint64_t oracle_pairing_pattern(uint64_t params_seed, uint64_t epoch,
                                uint64_t n, const uint32_t *offs,
                                const uint32_t *tgts, uint32_t *s) {
  uint32_t *order = (uint32_t *)malloc(n * sizeof(uint32_t));
  char *used = (char *)calloc(n, 1);
  for (uint64_t i = 0; i < n; i++) order[i] = (uint32_t)i;
  fisher_yates(params_seed, epoch, order, n);
  const uint64_t ek = oracle_seed(params_seed, epoch);
  uint64_t num = 0;
  for (uint64_t t = 0; t < n; t++) {
    uint32_t i = order[t];
    uint64_t len = offs[i + 1] - offs[i];
    if (len == 0) continue;
    uint64_t idx = oracle_seed(params_seed, ek ^ oracle_seed(params_seed, i)) % len;
    uint32_t neigh = tgts[offs[i] + idx];
    if (used[i] || used[neigh]) continue;
    used[i] = used[neigh] = 1;
    s[num * 2] = i;
    s[num * 2 + 1] = neigh;
    num++;
  }
  uint64_t idx = num * 2;
  for (uint64_t i = 0; i < n && idx < n; i++)
    if (!used[i]) s[idx++] = (uint32_t)i;
  free(order);
  free(used);
  return num;
}

/* ------------------------------------------------------------------------ */
/* MutateAndRunPrograms (common_language.h:157-193). */

uint64_t oracle_mutate_and_run(int lang, uint8_t *soup, const uint32_t *s,
                               uint64_t epoch_key, uint32_t mutation_prob,
                               uint64_t n, uint64_t num_indices, int nthreads,
                               uint64_t *raw_steps) {
  build_tables();
  uint64_t total = 0, total_raw = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total, total_raw) num_threads(nthreads)
  for (uint64_t k = 0; k < n / 2; k++) {
    uint8_t tape[PAIR];
    uint32_t p1 = s[2 * k], p2 = s[2 * k + 1];
    memcpy(tape, soup + (uint64_t)p1 * TAPE, TAPE);
    memcpy(tape + TAPE, soup + (uint64_t)p2 * TAPE, TAPE);
    for (uint64_t i = 0; i < PAIR; i++) {
      uint64_t r = oracle_splitmix64((n * epoch_key + k) * PAIR + i);
      if (((r >> 8) & ((1ULL << 30) - 1)) < mutation_prob) tape[i] = (uint8_t)r;
    }
    uint64_t raw = 0;
    if (k < num_indices) total += oracle_evaluate(lang, tape, STEP_LIMIT, &raw);
    total_raw += raw;
    memcpy(soup + (uint64_t)p1 * TAPE, tape, TAPE);
    memcpy(soup + (uint64_t)p2 * TAPE, tape + TAPE, TAPE);
  }
  if (raw_steps) *raw_steps = total_raw;
  return total;
}

/* ------------------------------------------------------------------------ */
/* The epoch loop of RunSimulation (common_language.h:432-596), minus the
 * callback statistics. */

int oracle_run_epochs(const oracle_sim *p, uint8_t *soup, uint64_t first_epoch,
                      uint64_t n_epochs, uint64_t *reset_index,
                      uint64_t *ops_per_epoch, uint64_t *raw_per_epoch) {
  const uint64_t n = p->num_programs;
  if (n == 0 || n % 2 != 0 || p->lang < 0 || p->lang >= ORC_NUM_LANGS) return -1;
  if (p->pairing == ORC_PAIR_FIXED && (n & (n - 1)) != 0) return -1;
  if (p->pairing == ORC_PAIR_PATTERN && (!p->pat_offs || !p->pat_tgts)) return -1;
  uint32_t *s = (uint32_t *)malloc(n * sizeof(uint32_t));
  if (!s) return -1;
  for (uint64_t e = first_epoch; e < first_epoch + n_epochs; e++) {
    uint64_t num_indices = n / 2;
    switch (p->pairing) {
      case ORC_PAIR_SHUFFLE: oracle_pairing_shuffle(p->seed, e, n, s); break;
      case ORC_PAIR_FIXED: oracle_pairing_fixed(e, n, s); break;
      case ORC_PAIR_CYCLIC: oracle_pairing_cyclic(e, n, s); break;
      default:
        num_indices = oracle_pairing_pattern(p->seed, e, n, p->pat_offs, p->pat_tgts, s);
    }
    uint64_t raw = 0;
    uint64_t ops = oracle_mutate_and_run(p->lang, soup, s, oracle_seed(p->seed, e),
                                         p->mutation_prob, n, num_indices,
                                         p->nthreads, &raw);
    if (ops_per_epoch) ops_per_epoch[e - first_epoch] = ops;
    if (raw_per_epoch) raw_per_epoch[e - first_epoch] = raw;
    /* common_language.h:590-595: reset after the epoch's callback; the grid
     * there covers only the first (n / 32) * 32 programs. */
    if (p->reset_interval && e % p->reset_interval == 0) {
      oracle_init_programs(oracle_seed(p->seed, *reset_index), n, soup,
                           p->zero_init, (n / 32) * 32);
      (*reset_index)++;
    }
  }
  free(s);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* CheckSelfRep (common_language.h:203-277). */

void oracle_check_selfrep(int lang, const uint8_t *soup, uint64_t epoch_key,
                          uint64_t n, uint64_t count, uint64_t *result,
                          int nthreads) {
  build_tables();
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
  for (uint64_t index = 0; index < count; index++) {
    enum { ITERS = 13, GENS = 4 };
    uint8_t tapes[ITERS][PAIR];
    const uint8_t *prog = soup + index * TAPE;
    uint64_t local_seed = oracle_splitmix64(n * epoch_key + index);
    for (uint64_t it = 0; it < ITERS; it++) {
      uint8_t noise[TAPE];
      for (int j = 0; j < TAPE; j++)
        noise[j] = (uint8_t)oracle_splitmix64(
            local_seed ^ oracle_splitmix64((it + 1) * TAPE + (uint64_t)j));
      uint8_t *t = tapes[it];
      memcpy(t, prog, TAPE);
      memcpy(t + TAPE, noise, TAPE);
      oracle_evaluate(lang, t, STEP_LIMIT, NULL);
      for (int g = 0; g < GENS; g++) {
        memcpy(t, t + TAPE, TAPE);
        memcpy(t + TAPE, noise, TAPE);
        oracle_evaluate(lang, t, STEP_LIMIT, NULL);
      }
    }
    uint64_t res[2] = {0, 0};
    for (int i = 0; i < PAIR; i++) {
      for (int a = 0; a < ITERS; a++) {
        uint64_t cnt = 1;
        if (i < TAPE && tapes[a][i] != prog[i]) continue;
        for (int b = a + 1; b < ITERS; b++)
          if (tapes[a][i] == tapes[b][i]) cnt++;
        if (cnt > ITERS / 4) {
          res[i / TAPE]++;
          break;
        }
      }
    }
    result[index] = res[0] < res[1] ? res[0] : res[1];
  }
}
