/*
 * clrun.h -- the reference's device-boundary API (src/clrun.h:25-30),
 * kept call for call so that the reference's drivers (rootsearch,
 * perft, selftest, benchmark: src/search.c, src/test.c, src/bench.c)
 * drive the GB300 kernels unchanged.  Implemented over libzeta_cuda.so
 * by zeta_gb300/host/cudarun.c; data moves through the globals declared
 * in zeta_gb300/host/engine.h, as it does through src/zeta.h:35-139.
 *
 * Every call returns true on success; on failure it prints the library's
 * error text to stderr (and to the log when logging is on), as
 * print_debug does (src/clrun.c:1492-1506).
 */
#ifndef ZETA_CLRUN_H
#define ZETA_CLRUN_H

#include <stdbool.h>
#include <stdint.h>

/* kernelname: "alphabeta_gpu" or "perft_gpu" (src/clrun.c:51-514).
 * Allocates the transposition tables of tt1_memory / tt2_memory MB. */
bool cl_init_device(char *kernelname);
/* stage the launch inputs: board, zeroed counters, hash history, random
 * numbers (src/clrun.c:516-673) */
bool cl_write_objects(void);
/* one search launch to `depth` with a node budget (src/clrun.c:675-974) */
bool cl_run_alphabeta(bool stm, int32_t depth, uint64_t nodes);
/* one perft launch to `depth` (src/clrun.c:979-1147) */
bool cl_run_perft(bool stm, int32_t depth);
/* results into COUNTERS and PV (src/clrun.c:1150-1266) */
bool cl_read_memory(void);
/* free the device state (src/clrun.c:1268-1490) */
bool cl_release_device(void);

#endif
