/*
 * engine.h -- globals and drivers of the zeta host (the reference keeps
 * the same state in src/zeta.h:35-139 and drives the device from
 * src/search.c, src/test.c, src/xboard.c).
 */
#ifndef ZETA_HOST_ENGINE_H
#define ZETA_HOST_ENGINE_H

#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/clrun.h"
#include "board.h"

/* engine state (src/zeta.h) */
extern Bitboard BOARD[7];
extern int STM;
extern int SD;                 /* max search depth */
extern int PLY;                /* game plies since setboard */
extern int GAMEPLY;
extern Bitboard HashHistory[MAXGAMEPLY];
extern Move MoveHistory[MAXGAMEPLY];

/* device-boundary staging (what cl_write_objects/cl_read_memory move):
 * GLOBAL_BOARD, COUNTERS, PV, GLOBAL_HASHHISTORY and the configuration
 * globals are declared by include/clrun.h with the reference's types */
extern uint32_t *RNUMBERS;

/* configuration (config.txt keys, src/io.c:533-583) */
extern uint64_t MaxNodes;

/* time control (src/zeta.c:78-85): timemode 0 = fixed time per move
 * (`st`), 1 = conventional clock (`level` with moves per session), 2 =
 * incremental clock (`level 0 ...`); times in milliseconds */
extern int timemode, MovesLeft, MaxMoves;
extern double TimeInc, TimeBase, TimeLeft, MaxTime;

/* results */
extern uint64_t ABNODECOUNT, TTHITS, TTSCOREHITS, IIDHITS;


bool read_config(const char *path);
bool engine_alloc(void);
void engine_free(void);
double get_time_ms(void);

/* drivers */
void perft(Bitboard *board, int stm, int depth);             /* src/search.c:225-271 */
Move rootsearch(Bitboard *board, int stm, int depth);        /* src/search.c:35-223 */
int selftest(void);                                          /* src/test.c:36-169 */
void benchsmp(Bitboard *board, int stm, int depth, uint64_t max_workers); /* src/xboard.c:822-974 */
int benchfile(const char *path, int depth, uint64_t max_workers); /* src/xboard.c:975-1428, list from a file */
void xboard(void);                                           /* src/xboard.c:44-1499 */

#endif
