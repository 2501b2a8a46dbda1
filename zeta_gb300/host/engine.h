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

#include "board.h"

/* engine state (src/zeta.h) */
extern Bitboard BOARD[7];
extern int STM;
extern int SD;                 /* max search depth */
extern int PLY;                /* game plies since setboard */
extern int GAMEPLY;
extern Bitboard HashHistory[MAXGAMEPLY];
extern Move MoveHistory[MAXGAMEPLY];

/* device-boundary staging (what cl_write_objects/cl_read_memory move) */
extern Bitboard GLOBAL_BOARD[7];
extern uint64_t *COUNTERS;       /* totalWorkUnits * 64 */
extern uint32_t *PV;             /* MAXPLY: PV[0] score, PV[1..] moves */
extern uint64_t *GLOBAL_HASHHISTORY;
extern uint32_t *RNUMBERS;

/* configuration (config.txt keys, src/io.c:533-583) */
extern uint64_t threadsX, threadsY, totalWorkUnits;
extern uint64_t tt1_memory, tt2_memory;
extern int64_t nodes_per_second;
extern uint64_t MaxNodes;
extern int device_id;
extern int search_mode;          /* 1 the reference's search (default), 0 pure fixed-depth */

/* results */
extern uint64_t ABNODECOUNT, TTHITS, TTSCOREHITS, IIDHITS;

extern FILE *LogFile;

bool read_config(const char *path);
bool engine_alloc(void);
void engine_free(void);
double get_time_ms(void);

/* drivers */
void perft(Bitboard *board, int stm, int depth);             /* src/search.c:225-271 */
Move rootsearch(Bitboard *board, int stm, int depth);        /* src/search.c:35-223 */
int selftest(void);                                          /* src/test.c:36-169 */
void benchsmp(Bitboard *board, int stm, int depth, uint64_t max_workers); /* src/xboard.c:822-974 */
void xboard(void);                                           /* src/xboard.c:44-1499 */

#endif
