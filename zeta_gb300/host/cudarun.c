/*
 * cudarun.c -- the reference's device-boundary API (include/clrun.h;
 * src/clrun.c, src/clconfig.c, src/clquery.c) implemented over
 * libzeta_cuda.so.  The calls keep their names, their binary interface
 * (4-byte cl_bool), their data-in-globals contract and their synchronous
 * behaviour; the OpenCL context, program build and buffer plumbing of the
 * reference become zeta_init / zeta_perft / zeta_engine_search.  Linked
 * both into this project's host and, unchanged, into the reference's own
 * host.  No CPU fallback: when the library cannot run on a GB300 every
 * call returns false.
 */
#include <inttypes.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/clrun.h"
#include "../../include/zeta_cuda.h"

static int g_inited = 0;
static int g_pure = 0;
static int g_all_promotions = 0;

/* print_debug, src/clrun.c:1492-1506 */
static clrun_bool fail(const char *what) {
  fprintf(stderr, "Error: %s: %s\n", what, zeta_last_error());
  if (LogFile) fprintf(LogFile, "Error: %s: %s\n", what, zeta_last_error());
  return 0;
}

void cl_set_pure_search(int on) { g_pure = on != 0; }

void cl_set_all_promotions(int on) {
  g_all_promotions = on != 0;
  if (g_inited) zeta_perft_set_promotions(g_all_promotions);
}

clrun_bool cl_init_device(char *kernelname) {
  if (g_inited) cl_release_device();
  if (!kernelname || (strcmp(kernelname, "alphabeta_gpu") && strcmp(kernelname, "perft_gpu"))) {
    fprintf(stderr, "Error: unknown kernel %s\n", kernelname ? kernelname : "(null)");
    return 0;
  }
  /* the transposition tables come up zeroed, as the reference creates
   * them from zeroed host images (src/clrun.c:404-443) */
  if (zeta_init(opencl_device_id, tt1_memory, tt2_memory) != ZETA_OK) return fail("zeta_init");
  g_inited = 1;
  if (zeta_perft_set_promotions(g_all_promotions) != ZETA_OK) return fail("zeta_perft_set_promotions");
  return 1;
}

clrun_bool cl_write_objects(void) {
  /* the inputs stay in the host globals; each launch hands them to the
   * library (which stages them in pinned memory) */
  return g_inited ? 1 : 0;
}

clrun_bool cl_run_perft(clrun_bool stm, int32_t depth) {
  if (!g_inited) return 0;
  uint64_t leaves = 0;
  if (zeta_perft(GLOBAL_BOARD, stm ? 1 : 0, depth, &leaves) != ZETA_OK) return fail("zeta_perft");
  /* worker 0 reports the leaf count in counter slot 1 (zetaperft.cl:1319) */
  memset(COUNTERS, 0, totalWorkUnits * 64 * sizeof(uint64_t));
  COUNTERS[1] = leaves;
  return 1;
}

clrun_bool cl_run_alphabeta(clrun_bool stm, int32_t depth, uint64_t nodes) {
  if (!g_inited) return 0;
  const int workers = totalWorkUnits < 1 ? 1 : (int)totalWorkUnits;
  if (g_pure && depth >= 1) {
    /* pure fixed-depth search (no reference counterpart): root = negamax */
    memset(COUNTERS, 0, totalWorkUnits * 64 * sizeof(uint64_t));
    if (zeta_search(GLOBAL_BOARD, stm ? 1 : 0, depth, PLY, GLOBAL_HASHHISTORY, nodes, PV, COUNTERS) != ZETA_OK)
      return fail("zeta_search");
    return 1;
  }
  /* the reference's search: totalWorkUnits workers, COUNTERS per worker;
   * the hash history is replicated per worker by the host, worker 0's copy
   * is the game's (src/search.c:50-54) */
  if (zeta_engine_search(GLOBAL_BOARD, stm ? 1 : 0, depth, PLY, GLOBAL_HASHHISTORY, nodes, workers, PV, COUNTERS) !=
      ZETA_OK)
    return fail("zeta_engine_search");
  return 1;
}

clrun_bool cl_read_memory(void) {
  /* zeta_perft / zeta_engine_search returned their results synchronously */
  return g_inited ? 1 : 0;
}

clrun_bool cl_release_device(void) {
  if (!g_inited) return 1;
  g_inited = 0;
  if (zeta_release() != ZETA_OK) return fail("zeta_release");
  return 1;
}

/* ------------------------------------------------------------------ */
/* -pl / -dl (src/clquery.c:33-325): one CUDA platform, its devices. */
clrun_bool cl_platform_list(void) {
  printf("#> ### Platform 0: CUDA (libzeta_cuda, sm_103a kernels)\n");
  return 1;
}

clrun_bool cl_device_list(void) {
  int sms = 0, major = 0, minor = 0;
  uint64_t hbm = 0;
  if (zeta_device_info(&sms, &major, &minor, &hbm) != ZETA_OK) return fail("zeta_device_info");
  printf("#> ### Device %d: compute capability %d.%d, %d SMs, %" PRIu64 " MB device memory\n", opencl_device_id,
         major, minor, sms, hbm >> 20);
  return 1;
}

/* ------------------------------------------------------------------ */
/* --guessconfig / --guessconfigx (src/clconfig.c:33-1058).  The
 * reference sizes its tables from the device's allocation limits, then
 * doubles threadsY while a node-rate benchmark improves by at least
 * SPEEDUPMARGIN (1.68, src/types.h:82).  A node rate keeps rising with
 * more workers long after the time to depth stops falling (more workers
 * search a larger tree), so this tuner measures what a game uses: the time
 * of the reference's iterative deepening from the initial position with
 * fresh tables, for a doubling worker count, and keeps the fastest.
 * --guessconfig: depth 9, one run per count, 16..512 workers;
 * --guessconfigx: depth 11, the median of three runs, 16..2048 workers.
 * The result is written to config.txt in the reference's key format
 * (threadsX x threadsY = workers, nodes_per_second, table sizes, device). */
static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + (double)t.tv_nsec * 1e-9;
}

/* the initial position, as src/io.c setboard leaves it */
static const uint64_t kStartBoard[7] = {0xFFFF000000000000ULL, 0x91FF00000000FF91ULL, 0x5A0000000000005AULL,
                                        0xAD000000000000ADULL, 0x6EFFFFFFFFFFFF6EULL, 0x18892007F9451009ULL, 0};

static int time_to_depth(int depth, int workers, double *secs, uint64_t *nodes) {
  if (zeta_tt_clear() != ZETA_OK) return 0;
  uint8_t stm = 0, done = 0;
  int32_t score = 0;
  uint32_t move = 0;
  uint64_t n = 0;
  double t0 = now_s();
  if (zeta_engine_id(kStartBoard, &stm, 1, depth, workers, 0, 0, &score, &move, &n, &done, NULL, NULL, NULL) !=
      ZETA_OK)
    return 0;
  *secs = now_s() - t0;
  *nodes = n;
  return 1;
}

static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

clrun_bool cl_guess_config(clrun_bool extreme) {
  int sms = 0, major = 0, minor = 0;
  uint64_t hbm = 0;
  const int depth = extreme ? 11 : 9, reps = extreme ? 3 : 1, wmax = extreme ? 2048 : 512;
  /* tables: TT1 of up to 8 GB, an eighth of the device memory; TT2 off --
   * on this device the helpers share TT1 alone and reach depth sooner
   * than with the ABDADA locks of TT2 */
  uint64_t t1 = 0;
  int best_w = 1;
  double best_s = 1e30;
  uint64_t best_nps = 0;
  if (g_inited) cl_release_device();
  if (zeta_init(opencl_device_id, 0, 0) != ZETA_OK || zeta_device_info(&sms, &major, &minor, &hbm) != ZETA_OK)
    return fail("zeta_init");
  zeta_release();
  t1 = hbm / 8 >> 20;
  if (t1 > 8192) t1 = 8192;
  if (zeta_init(opencl_device_id, t1, 0) != ZETA_OK) return fail("zeta_init");
  printf("#> ### guessing config: device %d, %d SMs, TT1 %" PRIu64 " MB, time to depth %d from the initial "
         "position ###\n", opencl_device_id, sms, t1, depth);
  for (int w = 16; w <= wmax; w *= 2) {
    double runs[3];
    uint64_t nodes = 0, n = 0;
    for (int r = 0; r < reps; r++) {
      if (!time_to_depth(depth, w, &runs[r], &n)) {
        zeta_release();
        return fail("zeta_engine_id");
      }
      nodes += n;
    }
    qsort(runs, (size_t)reps, sizeof runs[0], cmp_double);
    const double med = runs[reps / 2];
    const uint64_t nps = (uint64_t)((double)nodes / reps / med);
    printf("#> workers %5d: %8.3f s to depth %d, %" PRIu64 " nps\n", w, med, depth, nps);
    if (med < best_s) {
      best_s = med;
      best_w = w;
      best_nps = nps;
    }
  }
  zeta_release();
  char note[128];
  snprintf(note, sizeof note, "CUDA device %d (compute capability %d.%d, %d SMs)", opencl_device_id, major, minor,
           sms);
  if (!clrun_write_config("config.txt", (uint64_t)best_w, best_nps, t1, 0, opencl_device_id, note)) {
    fprintf(stderr, "Error: cannot write config.txt\n");
    return 0;
  }
  printf("#> ### config.txt written: %d workers, %.3f s to depth %d ###\n", best_w, best_s, depth);
  return 1;
}

/* config.txt in the reference's key format (src/clconfig.c:784-804, read
 * back by src/io.c:533-583): threadsX x threadsY workers, node rate, table
 * sizes, device */
clrun_bool clrun_write_config(const char *path, uint64_t workers, uint64_t nps, uint64_t tt1_mb, uint64_t tt2_mb,
                              int32_t device, const char *note) {
  FILE *cfg = fopen(path, "w");
  if (!cfg) return 0;
  fprintf(cfg, "################################################################################\n");
  fprintf(cfg, "// Zeta config file for %s\n", note ? note : "a CUDA device");
  fprintf(cfg, "################################################################################\n");
  fprintf(cfg, "threadsX: %" PRIu64 ";\n", workers);
  fprintf(cfg, "threadsY: %d;\n", 1);
  fprintf(cfg, "nodes_per_second: %" PRIu64 ";\n", nps);
  fprintf(cfg, "tt1_memory: %" PRIu64 "; // in MB\n", tt1_mb);
  fprintf(cfg, "tt2_memory: %" PRIu64 "; // in MB\n", tt2_mb);
  fprintf(cfg, "opencl_platform_id: %d;\n", 0);
  fprintf(cfg, "opencl_device_id: %d;\n", device);
  fprintf(cfg, "opencl_gpugen: %d;\n", 0);
  fprintf(cfg, "################################################################################\n");
  fprintf(cfg, "# threadsX           // search workers (threadsX x threadsY)\n");
  fprintf(cfg, "# threadsY           // multiplier for threadsX\n");
  fprintf(cfg, "# nodes_per_second   // nps of device, for initial time control\n");
  fprintf(cfg, "# tt1_memory         // MB of device memory for the classic hash table\n");
  fprintf(cfg, "# tt2_memory         // MB of device memory for the ABDADA hash table\n");
  fprintf(cfg, "# opencl_device_id   // CUDA device ordinal\n");
  fprintf(cfg, "################################################################################\n");
  return fclose(cfg) == 0 ? 1 : 0;
}
