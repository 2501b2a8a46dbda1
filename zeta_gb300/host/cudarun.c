/*
 * cudarun.c -- the reference's device-boundary API (include/clrun.h,
 * src/clrun.c) implemented over libzeta_cuda.so.  The six calls keep
 * their names, their data-in-globals contract and their synchronous
 * behaviour; the OpenCL context, program build and buffer plumbing of the
 * reference become zeta_init / zeta_perft / zeta_search.  No CPU fallback:
 * when the library cannot run on a GB300 every call returns false.
 */
#include <stdio.h>
#include <string.h>

#include "../../include/clrun.h"
#include "../../include/zeta_cuda.h"
#include "engine.h"

static bool g_inited = false;
static char g_kernel[32] = "";

/* print_debug, src/clrun.c:1492-1506 */
static bool fail(const char *what) {
  fprintf(stderr, "Error: %s: %s\n", what, zeta_last_error());
  if (LogFile) fprintf(LogFile, "Error: %s: %s\n", what, zeta_last_error());
  return false;
}

bool cl_init_device(char *kernelname) {
  if (g_inited) cl_release_device();
  if (strcmp(kernelname, "alphabeta_gpu") && strcmp(kernelname, "perft_gpu")) {
    fprintf(stderr, "Error: unknown kernel %s\n", kernelname);
    return false;
  }
  /* the transposition tables come up zeroed, as the reference creates
   * them from zeroed host images (src/clrun.c:404-443) */
  if (zeta_init(device_id, tt1_memory, tt2_memory) != ZETA_OK) return fail("zeta_init");
  snprintf(g_kernel, sizeof g_kernel, "%s", kernelname);
  g_inited = true;
  return true;
}

bool cl_write_objects(void) {
  /* the inputs stay in the host globals; each launch hands them to the
   * library (which stages them in pinned memory) */
  return g_inited;
}

bool cl_run_perft(bool stm, int32_t depth) {
  if (!g_inited) return false;
  uint64_t leaves = 0;
  if (zeta_perft(GLOBAL_BOARD, stm ? 1 : 0, depth, &leaves) != ZETA_OK) return fail("zeta_perft");
  /* worker 0 reports the leaf count in counter slot 1 (zetaperft.cl:1319) */
  memset(COUNTERS, 0, totalWorkUnits * 64 * sizeof(uint64_t));
  COUNTERS[1] = leaves;
  return true;
}

bool cl_run_alphabeta(bool stm, int32_t depth, uint64_t nodes) {
  if (!g_inited) return false;
  if (search_mode == 0) {
    /* pure fixed-depth search (no reference counterpart): root = negamax */
    memset(COUNTERS, 0, totalWorkUnits * 64 * sizeof(uint64_t));
    if (zeta_search(GLOBAL_BOARD, stm ? 1 : 0, depth, PLY, GLOBAL_HASHHISTORY, nodes, PV, COUNTERS) != ZETA_OK)
      return fail("zeta_search");
    return true;
  }
  /* the reference's search: totalWorkUnits workers, COUNTERS per worker */
  if (zeta_engine_search(GLOBAL_BOARD, stm ? 1 : 0, depth, PLY, GLOBAL_HASHHISTORY, nodes, (int)totalWorkUnits, PV,
                         COUNTERS) != ZETA_OK)
    return fail("zeta_engine_search");
  return true;
}

bool cl_read_memory(void) {
  /* zeta_perft / zeta_search returned their results synchronously */
  return g_inited;
}

bool cl_release_device(void) {
  if (!g_inited) return true;
  g_inited = false;
  if (zeta_release() != ZETA_OK) return fail("zeta_release");
  return true;
}
