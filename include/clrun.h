/*
 * clrun.h -- the reference's device-boundary API (src/clrun.h:25-30) with
 * the reference's own binary interface, implemented over libzeta_cuda.so
 * by zeta_gb300/host/cudarun.c.
 *
 * The reference's host C (src/zeta.c, search.c, test.c, bench.c,
 * xboard.c, io.c, bitboard.c, bit.c, timer.c) links against cudarun.o and
 * libzeta_cuda.so in place of clrun.c, clconfig.c, clquery.c and the
 * OpenCL library, with no source change: the calls keep their names and
 * argument types, and the data moves through the reference's own globals
 * (src/zeta.h:35-139), which the host defines and cudarun.c reads.
 *
 * Types, as the reference defines them (src/types.h:30-37): its `bool` is
 * cl_bool = cl_uint, a 4-byte unsigned integer (here clrun_bool), s32 is
 * int32_t, u64 uint64_t, Bitboard / Hash uint64_t, Move uint32_t.
 *
 * Every call returns 1 on success; on failure it prints the library's
 * error text to stderr (and to LogFile when one is open), as print_debug
 * does (src/clrun.c:1492-1506), and returns 0.
 */
#ifndef ZETA_CLRUN_H
#define ZETA_CLRUN_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint32_t clrun_bool; /* cl_bool, src/types.h:37 */

/* src/clrun.h:25-30 */
/* kernelname: "alphabeta_gpu" or "perft_gpu" (src/clrun.c:51-514).
 * Brings up device opencl_device_id and its transposition tables of
 * tt1_memory / tt2_memory MB, zeroed. */
clrun_bool cl_init_device(char *kernelname);
/* stage the launch inputs: board, zeroed counters, hash history, random
 * numbers (src/clrun.c:516-673); the run calls read the globals directly */
clrun_bool cl_write_objects(void);
/* one search launch of totalWorkUnits workers to `depth` with a node
 * budget per worker (src/clrun.c:675-974); depth 0 is the start-up
 * warm-up of src/zeta.c:695 (a quiescence search of the root) */
clrun_bool cl_run_alphabeta(clrun_bool stm, int32_t depth, uint64_t nodes);
/* one perft launch to `depth` (src/clrun.c:979-1147) */
clrun_bool cl_run_perft(clrun_bool stm, int32_t depth);
/* results into COUNTERS and PV (src/clrun.c:1150-1266) */
clrun_bool cl_read_memory(void);
/* free the device state (src/clrun.c:1268-1490) */
clrun_bool cl_release_device(void);

/* src/clconfig.h:25 -- the reference's --guessconfig / --guessconfigx:
 * measure the search on the device and write config.txt (see cudarun.c) */
clrun_bool cl_guess_config(clrun_bool extreme);
/* src/clquery.h:25-26 -- the reference's -pl / -dl listings: here the one
 * CUDA platform and its devices */
clrun_bool cl_platform_list(void);
clrun_bool cl_device_list(void);

/* The file cl_guess_config writes: config.txt keys in the reference's
 * format (src/clconfig.c:784-804), which the reference's
 * read_and_init_config (src/io.c:533-583) and this project's host read
 * back.  Returns 1 on success. */
clrun_bool clrun_write_config(const char *path, uint64_t workers, uint64_t nps, uint64_t tt1_mb, uint64_t tt2_mb,
                              int32_t device, const char *note);

/* No counterpart in the reference: makes cl_run_alphabeta run the pure
 * fixed-depth search (root score = plain negamax) instead of the
 * reference's search with its heuristics (the default). */
void cl_set_pure_search(int on);

/* No counterpart in the reference: with on != 0, cl_run_perft lets a pawn
 * promote to a queen, rook, bishop or knight (four moves); the default is
 * the reference's queen-only rule (zetaperft.cl:1380-1384).  Kept across
 * cl_release_device / cl_init_device. */
void cl_set_all_promotions(int on);

/* The reference's globals that the calls above read and write, with the
 * reference's types (src/zeta.h:35-139; defined by the host, src/zeta.c). */
extern uint64_t *GLOBAL_BOARD;       /* Bitboard[7], the position to search */
extern uint64_t *COUNTERS;           /* totalWorkUnits x 64; slot 1 nodes / leaves */
extern uint32_t *PV;                 /* 64 Moves: PV[0] score, PV[1..] moves */
extern uint64_t *GLOBAL_HASHHISTORY; /* totalWorkUnits x 1024 game hashes */
extern int32_t PLY;                  /* game ply of the root (ply_init) */
extern uint64_t totalWorkUnits;      /* workers = threadsX * threadsY */
extern uint64_t threadsX, threadsY;
extern uint64_t tt1_memory, tt2_memory; /* MB */
extern int64_t nodes_per_second;
extern int32_t opencl_device_id;     /* the CUDA device ordinal */
extern FILE *LogFile;

#ifdef __cplusplus
}
#endif
#endif
