/*
 * engine.c -- host drivers of the device path: perft (src/search.c:225-271),
 * selftest (src/test.c:36-169) and iterative-deepening rootsearch
 * (src/search.c:35-223), all through the clrun.h calls.
 */
#include <inttypes.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/clrun.h"
#include "engine.h"

Bitboard BOARD[7];
int STM = WHITE, SD = MAXPLY - 1, PLY = 0, GAMEPLY = 0;
Bitboard HashHistory[MAXGAMEPLY];
Move MoveHistory[MAXGAMEPLY];
Bitboard *GLOBAL_BOARD = NULL;
uint64_t *COUNTERS = NULL;
uint32_t *PV = NULL;
uint64_t *GLOBAL_HASHHISTORY = NULL;
uint32_t *RNUMBERS = NULL;
uint64_t threadsX = 1, threadsY = 1, totalWorkUnits = 1;
uint64_t tt1_memory = 256, tt2_memory = 0;
int64_t nodes_per_second = 1000000;
uint64_t MaxNodes = 0;
int timemode = 0, MovesLeft = 1, MaxMoves = 1;
double TimeInc = 0, TimeBase = 5 * 1000, TimeLeft = 5 * 1000, MaxTime = 5 * 1000;
int32_t opencl_device_id = 0;
uint64_t ABNODECOUNT = 0, TTHITS = 0, TTSCOREHITS = 0, IIDHITS = 0;
FILE *LogFile = NULL;

double get_time_ms(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec * 1000.0 + t.tv_nsec / 1e6;
}

/* read_and_init_config, src/io.c:533-583: the same keys; a missing file
 * keeps the defaults (one worker, 256 MB table) */
bool read_config(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) return false;
  char line[1024];
  while (fgets(line, sizeof line, f)) {
    sscanf(line, "threadsX: %" SCNu64 ";", &threadsX);
    sscanf(line, "threadsY: %" SCNu64 ";", &threadsY);
    sscanf(line, "nodes_per_second: %" SCNi64 ";", &nodes_per_second);
    sscanf(line, "tt1_memory: %" SCNu64 ";", &tt1_memory);
    sscanf(line, "tt2_memory: %" SCNu64 ";", &tt2_memory);
    sscanf(line, "opencl_device_id: %d;", &opencl_device_id);
    sscanf(line, "device_id: %d;", &opencl_device_id);
  }
  fclose(f);
  MaxNodes = (uint64_t)nodes_per_second;
  totalWorkUnits = threadsX * threadsY;
  if (totalWorkUnits < 1) totalWorkUnits = 1;
  return true;
}

bool engine_alloc(void) {
  GLOBAL_BOARD = calloc(7, sizeof(Bitboard));
  COUNTERS = calloc(totalWorkUnits * 64, sizeof(uint64_t));
  PV = calloc(MAXPLY, sizeof(uint32_t));
  GLOBAL_HASHHISTORY = calloc(totalWorkUnits * MAXGAMEPLY, sizeof(uint64_t));
  RNUMBERS = calloc(totalWorkUnits * 64, sizeof(uint32_t));
  return GLOBAL_BOARD && COUNTERS && PV && GLOBAL_HASHHISTORY && RNUMBERS;
}

void engine_free(void) {
  free(GLOBAL_BOARD);
  free(COUNTERS);
  free(PV);
  free(GLOBAL_HASHHISTORY);
  free(RNUMBERS);
  GLOBAL_BOARD = NULL;
  COUNTERS = NULL;
  PV = NULL;
  GLOBAL_HASHHISTORY = NULL;
  RNUMBERS = NULL;
}

static void die(void) {
  cl_release_device();
  engine_free();
  exit(EXIT_FAILURE);
}

void perft(Bitboard *board, int stm, int depth) {
  ABNODECOUNT = 0;
  memcpy(GLOBAL_BOARD, board, 7 * sizeof(Bitboard));
  memset(COUNTERS, 0, totalWorkUnits * 64 * sizeof(uint64_t));
  for (uint64_t i = 0; i < totalWorkUnits; i++)
    memcpy(&GLOBAL_HASHHISTORY[i * MAXGAMEPLY], HashHistory, sizeof HashHistory);
  if (!cl_write_objects() || !cl_run_perft(stm, depth) || !cl_read_memory()) die();
  for (uint64_t i = 0; i < totalWorkUnits; i++) ABNODECOUNT += COUNTERS[i * 64 + 1];
}

/* One worker sweep: the iterative-deepening search of `board` to `depth`
 * with 1, 2, 4, ... workers up to max_workers, each run from fresh tables;
 * times (s), node rates and worker counts into the arrays (kMaxRuns long),
 * returns the number of runs. */
enum { kMaxRuns = 40 };
static int worker_sweep(Bitboard *board, int stm, int depth, uint64_t max_workers, const char *name, double *secs,
                        uint64_t *nps, uint64_t *workers) {
  int runs = 0;
  if (max_workers < 1) max_workers = 1;
  for (uint64_t w = 1; runs < kMaxRuns;) {
    printf("### doing inits for %s depth %d: ###\n", name, depth);
    totalWorkUnits = w;
    engine_free();
    if (!engine_alloc()) die();
    if (!cl_release_device() || !cl_init_device("alphabeta_gpu")) die(); /* fresh tables */
    printf("### computing %s depth %d: ###\n", name, depth);
    printf("### work-groups: %" PRIu64 " ###\n", w);
    double t0 = get_time_ms();
    rootsearch(board, stm, depth);
    double el = (get_time_ms() - t0 + 1.0) / 1000.0;
    secs[runs] = el;
    nps[runs] = (uint64_t)((double)ABNODECOUNT / el);
    workers[runs] = w;
    runs++;
    if (w >= max_workers) break;
    w = w * 2 > max_workers ? max_workers : w * 2;
  }
  return runs;
}

/* the results.txt table (src/xboard.c:923-944) */
static void scaling_table(int runs, const double *secs, const uint64_t *nps, const uint64_t *workers) {
  printf("### workers\t#nps\t\t#nps speedup\t#time in s\t#ttd speedup \t#relative ttd speedup ###\n");
  for (int i = 0; i < runs; i++) {
    const double ns = nps[0] ? (double)nps[i] / (double)nps[0] : 0.0;
    const double ttd = secs[0] / secs[i], rel = i ? secs[i - 1] / secs[i] : 1.0;
    printf("### %" PRIu64 "\t\t%" PRIu64 "\t\t%lf\t%lf\t%lf\t%lf \n", workers[i], nps[i], ns, secs[i], ttd, rel);
    if (LogFile)
      fprintf(LogFile, "### %" PRIu64 "\t\t%" PRIu64 "\t\t%lf\t%lf\t%lf\t%lf \n", workers[i], nps[i], ns, secs[i],
              ttd, rel);
  }
}

/* a depth-limited benchmark runs without node or time budget; the caller's
 * budgets, worker count and tables come back afterwards */
static uint64_t g_saved_workers, g_saved_nodes;
static double g_saved_time;
static void bench_begin(void) {
  g_saved_workers = totalWorkUnits;
  g_saved_nodes = MaxNodes;
  g_saved_time = MaxTime;
  MaxNodes = 0;
  MaxTime = 1e15;
}
static void bench_end(void) {
  totalWorkUnits = g_saved_workers;
  MaxNodes = g_saved_nodes;
  MaxTime = g_saved_time;
  engine_free();
  if (!engine_alloc()) die();
  if (!cl_release_device() || !cl_init_device("alphabeta_gpu")) die();
  fflush(stdout);
}

/* Worker-scaling benchmark (the reference's `benchsmp`, src/xboard.c:822-974):
 * the same iterative-deepening search to `depth` with 1, 2, 4, ... workers
 * up to max_workers, each run from fresh tables, then one table of nodes
 * per second, time-to-depth and the speedups over 1 worker and over the
 * previous worker count, in the reference's results.txt layout. */
void benchsmp(Bitboard *board, int stm, int depth, uint64_t max_workers) {
  double secs[kMaxRuns];
  uint64_t nps[kMaxRuns], workers[kMaxRuns];
  bench_begin();
  const int runs = worker_sweep(board, stm, depth, max_workers, "benchsmp", secs, nps, workers);
  scaling_table(runs, secs, nps, workers);
  bench_end();
}

/* The position-list benchmarks (the reference's `benchkaufmann` and
 * `benchhyatt24`, src/xboard.c:975-1200, 1203-1428): the worker sweep of
 * benchsmp on every position of a list, one table per position, then the
 * table of the times summed over the positions.  The reference embeds its
 * two lists (src/xboard.c:986-1012, 1214-1240); here the list is a file
 * of FEN lines, so any list -- those two included -- can be run. */
int benchfile(const char *path, int depth, uint64_t max_workers) {
  FILE *f = fopen(path, "r");
  if (!f) {
    printf("Error (cannot open %s): benchfile\n", path);
    return 0;
  }
  double secs[kMaxRuns], total[kMaxRuns] = {0};
  uint64_t nps[kMaxRuns], workers[kMaxRuns], nodes[kMaxRuns] = {0};
  int runs = 0, posi = 0;
  char line[1024];
  bench_begin();
  while (fgets(line, sizeof line, f)) {
    Bitboard b[7];
    int side, full;
    if (strlen(line) < 8 || line[0] == '#') continue;
    if (!board_setfen(b, &side, &full, line)) {
      printf("# Error (in setting fen position): %s", line);
      continue;
    }
    posi++;
    printf("#\n#\n### setting up board %d: ###\n", posi);
    memset(HashHistory, 0, sizeof HashHistory);
    HashHistory[0] = b[QBBHASH];
    runs = worker_sweep(b, side, depth, max_workers, "benchfile", secs, nps, workers);
    scaling_table(runs, secs, nps, workers);
    for (int i = 0; i < runs; i++) {
      total[i] += secs[i];
      nodes[i] += (uint64_t)((double)nps[i] * secs[i]);
    }
  }
  fclose(f);
  if (posi > 0) {
    printf("#\n### all %d positions: ###\n", posi);
    for (int i = 0; i < runs; i++) nps[i] = (uint64_t)((double)nodes[i] / total[i]);
    scaling_table(runs, total, nps, workers);
  }
  bench_end();
  return posi;
}

/* The 14 known-answer tests of the reference's selftest (src/test.c:43-73). */
int selftest(void) {
  static const char *fens[4] = {
      "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq -",
      "8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - -",
      "r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq -",
      "r4rk1/1pp1qppp/p1np1n2/2b1p1B1/2B1P1b1/P1NP1N2/1PP1QPPP/R4RK1 w - -"};
  static const struct { int fen, depth; uint64_t count; } kat[14] = {
      {0, 1, 20}, {0, 2, 400}, {0, 3, 8902}, {0, 4, 197281}, {1, 1, 14}, {1, 2, 191}, {1, 3, 2812},
      {1, 4, 43238}, {2, 1, 48}, {2, 2, 2039}, {2, 3, 97862}, {3, 1, 46}, {3, 2, 2079}, {3, 3, 89890}};
  if (!cl_release_device() || !cl_init_device("perft_gpu")) die();
  int passed = 0;
  for (int i = 0; i < 14; i++) {
    Bitboard b[7];
    int stm, full;
    printf("#> doing perft depth: %d for position %d of 14\n", kat[i].depth, i + 1);
    if (!board_setfen(b, &stm, &full, fens[kat[i].fen])) {
      printf("# Error (in setting fen position): setboard\n");
      continue;
    }
    double t0 = get_time_ms();
    perft(b, stm, kat[i].depth);
    double s = (get_time_ms() - t0) / 1000.0 + 1e-9;
    if (ABNODECOUNT == kat[i].count) {
      passed++;
      printf("#> OK, Nodecount Correct, %" PRIu64 " nodes in %lf seconds with %" PRIu64 " nps.\n", ABNODECOUNT, s,
             (uint64_t)(ABNODECOUNT / s));
    } else {
      printf("#> Error, Nodecount NOT Correct, %" PRIu64 " computed nodes != %" PRIu64 " nodes for depth %d.\n",
             ABNODECOUNT, kat[i].count, kat[i].depth);
    }
  }
  printf("#\n###############################\n### passed %d from 14 tests ###\n###############################\n",
         passed);
  if (!cl_release_device() || !cl_init_device("alphabeta_gpu")) die();
  return passed;
}

/* Iterative deepening, one launch per depth, the table kept between them
 * (src/search.c:35-223).  Prints "depth score time nodes pv" lines.
 * Budgets, as the reference's loop (src/search.c:194-198): a launch stops
 * when worker 0 has made MaxNodes / totalWorkUnits moves, and no deeper
 * iteration starts once the nodes so far times the estimated branching
 * factor (ESTEBF) exceed MaxNodes, or the time so far times ESTEBF exceeds
 * MaxTime.  (The reference compares seconds with MaxTime's milliseconds
 * there, which leaves only its node budget in force; both are in force
 * here.)  Once a node rate has been measured, a launch's node budget is
 * also capped at what that rate covers in the time left, so a fixed time
 * per move (`st`) holds even when nodes_per_second is not calibrated. */
Move rootsearch(Bitboard *board, int stm, int depth) {
  Move best = MOVENONE;
  int score = 0;
  double start = get_time_ms();
  ABNODECOUNT = TTHITS = TTSCOREHITS = IIDHITS = 0;
  memcpy(GLOBAL_BOARD, board, 7 * sizeof(Bitboard));
  for (uint64_t i = 0; i < totalWorkUnits; i++) {
    memcpy(&GLOBAL_HASHHISTORY[i * MAXGAMEPLY], HashHistory, sizeof HashHistory);
    for (int j = 0; j < 64; j++) RNUMBERS[i * 64 + j] = (uint32_t)rand();
  }
  /* 0 = no node budget, for depth-limited searches */
  const uint64_t max_nodes = MaxNodes ? MaxNodes : UINT64_MAX / ESTEBF;
  const uint64_t budget = max_nodes / totalWorkUnits;
  const double max_time_s = MaxTime / 1000.0;
  double el = 0.0;
  int idf = 1;
  do {
    uint64_t launch_budget = budget;
    if (idf > 1 && el > 0.005 && ABNODECOUNT > 0) {
      const double per_worker_rate = (double)ABNODECOUNT / el / (double)totalWorkUnits;
      const double left = max_time_s - el;
      const double cap = left > 0 ? left * per_worker_rate : 1.0;
      if (cap < (double)launch_budget) launch_budget = cap < 1.0 ? 1 : (uint64_t)cap;
    }
    memset(COUNTERS, 0, totalWorkUnits * 64 * sizeof(uint64_t));
    if (!cl_write_objects() || !cl_run_alphabeta(stm, idf, launch_budget) || !cl_read_memory()) die();
    for (uint64_t i = 0; i < totalWorkUnits; i++) {
      ABNODECOUNT += COUNTERS[i * 64 + 1];
      TTHITS += COUNTERS[i * 64 + 3];
      TTSCOREHITS += COUNTERS[i * 64 + 4];
      IIDHITS += COUNTERS[i * 64 + 5];
    }
    el = (get_time_ms() - start) / 1000.0;
    if (idf == 1 && JUSTMOVE(PV[1]) != MOVENONE) best = PV[1]; /* a move anyway */
    if (COUNTERS[1] < launch_budget) { /* not stopped by the node budget */
      if (JUSTMOVE(PV[1]) != MOVENONE) best = PV[1];
      score = ((int32_t)PV[0] == INF || (int32_t)PV[0] == -INF) ? 0 : (int32_t)PV[0];
      /* xboard mate scores, src/search.c:131-137 */
      int xs = score <= -MATESCORE ? -100000 - (INF + score) : score >= MATESCORE ? 100000 - (-INF + score) : score;
      if (JUSTMOVE(PV[1]) == MOVENONE) break;
      printf("%d %d %d %" PRIu64, idf, xs, (int)(el * 100), ABNODECOUNT);
      if (LogFile) fprintf(LogFile, "%d %d %d %" PRIu64, idf, xs, (int)(el * 100), ABNODECOUNT);
      for (int i = 1; i < MAXPLY && i <= idf && JUSTMOVE(PV[i]) != MOVENONE; i++) {
        char mv[6];
        move2can(PV[i], mv);
        printf(" %s", mv);
        if (LogFile) fprintf(LogFile, " %s", mv);
      }
      printf("\n");
      if (LogFile) fprintf(LogFile, "\n");
      fflush(stdout);
    } else if (launch_budget < budget) {
      break; /* stopped by the clock */
    }
    /* mate in n: no deeper iteration can change it (src/search.c:180-191) */
    if (score >= MATESCORE && score < INF && idf >= INF - score) break;
    if (score <= -MATESCORE && score > -INF && idf >= INF + score) break;
    idf++;
  } while (idf <= depth && el * ESTEBF < max_time_s && ABNODECOUNT * ESTEBF <= max_nodes && ABNODECOUNT > 1 &&
           idf < MAXPLY);
  return best;
}
