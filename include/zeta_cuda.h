/*
 * zeta_cuda.h -- C ABI of libzeta_cuda.so, the GB300 (sm_103a) device
 * path of the Zeta chess engine.
 *
 * The reference drives its OpenCL kernels through six calls that pass all
 * data in globals (src/clrun.h:25-30, src/zeta.h:35-139).  This library
 * exposes the same work as explicit calls with plain pointers and sizes;
 * include/clrun.h keeps the reference's six-call interface on top of it
 * (zeta_gb300/host/cudarun.c).
 *
 * Conventions
 *  - A board is the reference quad-bitboard, 7 x u64 (src/types.h:59-66):
 *    [0] black pieces, [1..3] piece-type planes, [4] moved flags (castle
 *    rights, en-passant target), [5] Zobrist hash, [6] half-move clock.
 *  - Moves are the reference's 32-bit packing (src/types.h:67-74).
 *  - Every call returns ZETA_OK (0) or a negative ZETA_ERR_* code; the
 *    text of the last error is in zeta_last_error().  No call falls back
 *    to the CPU: without a usable GB300 they fail.
 *  - One host thread drives the library (as src/clrun.c assumes).
 */
#ifndef ZETA_CUDA_H
#define ZETA_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZETA_OK 0
#define ZETA_ERR_CUDA -1       /* a CUDA runtime call failed */
#define ZETA_ERR_ARG -2        /* bad argument (size, depth, pointer) */
#define ZETA_ERR_STATE -3      /* zeta_init missing, or a second init */
#define ZETA_ERR_CAPACITY -4   /* a work buffer was too small */
#define ZETA_ERR_DEVICE -5     /* the kernel reported an error status */
#define ZETA_ERR_BUDGET -6     /* a bounded device loop gave up */
#define ZETA_ERR_NOALLOC -7    /* request exceeds a fixed-size static buffer */

/* ------------------------------------------------------------------ */
/* Device lifecycle.  Replaces cl_init_device / cl_release_device
 * (src/clrun.c:51-514, 1268-1490).  tt1_mb / tt2_mb size the two
 * transposition tables as the reference does (clrun.c:387-443: entries =
 * largest power of two that fits); 0 disables a table. */
int zeta_init(int device, uint64_t tt1_mb, uint64_t tt2_mb);
int zeta_release(void);
const char *zeta_last_error(void);

/* Device facts the autotuner and the bench report. */
int zeta_device_info(int *sm_count, int *cc_major, int *cc_minor, uint64_t *hbm_bytes);

/* ------------------------------------------------------------------ */
/* Perft (leaf count of the legal tree; promotions to a queen only, as the
 * reference generates them, unless zeta_perft_set_promotions(1)).
 * Replaces cl_run_perft (src/clrun.c:979-1147) + the COUNTERS read-back
 * and sum of src/search.c:225-271.  Host buffers. */
int zeta_perft(const uint64_t board[7], int stm, int depth, uint64_t *leaves);

/* n positions at once (one persistent work-stealing launch).
 * boards: n*7 u64, stm/depth: n bytes, leaves: n u64.  Host buffers. */
int zeta_perft_batch(const uint64_t *boards, const uint8_t *stm, const uint8_t *depth, int n,
                     uint64_t *leaves);

/* Same with DEVICE buffers already resident in HBM; enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and synchronised before
 * returning.  Used to time the kernels without host copies. */
int zeta_perft_batch_device(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth,
                            int n, uint64_t *d_leaves, void *stream);

/* Same work as zeta_perft_batch_device for callers that cannot allocate
 * device memory: programs that own every byte of device memory through
 * their own pool or budget, and latency-critical loops where a cudaMalloc
 * (which may synchronise the device) is not allowed.  No counterpart in
 * the reference.  It calls no cudaMalloc/cudaFree and needs no zeta_init:
 * its scratch is one fixed device array of about 29 MB inside the library,
 * held by every GPU that loads it until the process exits.
 *  - Limits: n <= 131072 positions, and the tree split may make at most
 *    131072 subtree tasks per level; beyond either it returns
 *    ZETA_ERR_NOALLOC.
 *  - The first call on a device looks up the array's device address (its
 *    host-side name is not a device address); that one-time set-up is
 *    serialised between host threads.
 *  - All calls share the one array: calls that overlap on the GPU (other
 *    streams, other host threads) race and give wrong counts.  Every call
 *    copies a status word back and synchronises `stream` before it
 *    returns, so a call cannot be captured into a CUDA graph.
 *  - Promotions follow zeta_perft_set_promotions, like the other entries. */
int zeta_perft_batch_noalloc(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n,
                             uint64_t *d_leaves, void *stream);

/* Launch geometry and split policy of the perft path (autotuner knobs).
 * threads_per_block: 64..1024, multiple of 32; blocks_per_sm: 0 = from
 * occupancy; min_tasks: split the tree until at least this many subtree
 * tasks exist (0 = 4 x resident threads); task_depth: remaining depth of a
 * subtree task, 1..4; use_graph: capture the launch sequence in a CUDA
 * graph and replay it while the shapes stay the same. */
typedef struct {
  int threads_per_block;
  int blocks_per_sm;
  uint32_t min_tasks;
  int task_depth;
  int use_graph;
} zeta_perft_config;
int zeta_perft_configure(const zeta_perft_config *cfg);
int zeta_perft_get_config(zeta_perft_config *cfg);

/* Promotion rule of every perft entry (zeta_perft, zeta_perft_batch,
 * zeta_perft_batch_device, zeta_perft_batch_noalloc): 0 (the default, and
 * the reference's rule, zetaperft.cl:1380-1384) a pawn reaching the last
 * rank becomes a queen; 1 it may become a queen, rook, bishop or knight
 * (four moves).  Lasts until changed or zeta_release.  No counterpart in
 * the reference.  Returns ZETA_ERR_ARG for other values;
 * zeta_perft_get_promotions gives the current rule. */
int zeta_perft_set_promotions(int all);
int zeta_perft_get_promotions(void);

/* Statistics of the last perft launch: subtree tasks, tasks taken from
 * another block's range, interior nodes generated, leaf-parent nodes
 * bulk-counted, device time of the work-stealing kernel (ms). */
typedef struct {
  uint64_t tasks;
  uint64_t steals;
  uint64_t interior_nodes;
  uint64_t counted_nodes;
  float kernel_ms;
  float total_ms;
} zeta_perft_stats;
int zeta_perft_last_stats(zeta_perft_stats *st);

/* ------------------------------------------------------------------ */
/* Batched fixed-depth search ("pure" alpha-beta): legal moves, the
 * reference evaluation (zeta.cl:1479-1554) at the leaves, mate -INF+ply,
 * stalemate 0, no quiescence/extensions/pruning/draw rules, so each root
 * score equals plain negamax.  `workers` ABDADA workers per position share
 * the transposition table (zeta_init's tt1, kept between calls; entries
 * are used only at equal remaining depth, so stale entries stay correct).
 * Replaces the fixed-depth use of cl_run_alphabeta (src/clrun.c:675-974)
 * for a batch.  Outputs: score from the side to move, a best move (one
 * that reaches the score), visited nodes summed over the workers. */
int zeta_search_batch(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, int32_t *scores,
                      uint32_t *bestmoves, uint64_t *nodes);
/* same with device buffers, on `stream` (NULL = the library's stream) */
int zeta_search_batch_device(const uint64_t *d_boards, const uint8_t *d_stm, int n, int depth, int workers,
                             int32_t *d_scores, uint32_t *d_bestmoves, uint64_t *d_nodes, void *stream);
/* One position to `depth` (cl_run_alphabeta, src/clrun.c:675-974, with
 * the read-back of src/clrun.c:1150-1266): pv[0] = root score, pv[1] =
 * best move; counters[1] = visited nodes.  ply_init, hash_history and
 * max_nodes carry the reference's arguments (game ply, repetition history
 * of MAXGAMEPLY hashes, node budget); the fixed-depth search does not
 * use them. */
int zeta_search(const uint64_t board[7], int stm, int depth, int ply_init, const uint64_t *hash_history,
                uint64_t max_nodes, uint32_t pv[64], uint64_t counters[64]);
/* Iterative deepening 1..depth of the batched pure search, the
 * transposition table kept between iterations (src/search.c:77-198).
 * ordering: 0 the hand-written ordering; 1 / 2 the move-ordering network
 * in BF16 / FP8 at nodes with >= 3 plies left -- every iteration is one
 * kernel step that logs the nodes without a network ordering, then one
 * batched tensor-core inference orders them for the next iteration.  No
 * counterpart in the reference (its ordering is hand-written,
 * zeta.cl:2039-2110).  Root scores do not depend on the ordering.  Host
 * buffers; nodes summed over the iterations; times in ms (wall, search
 * kernels, network). */
int zeta_search_id(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, int ordering,
                   int32_t *scores, uint32_t *bestmoves, uint64_t *nodes, float *ms_total, float *ms_search,
                   float *ms_net);
/* How the network's ordering enters the move order: its `top` best moves
 * (1..12) are searched right after the transposition-table move
 * (quiet_only = 0), or they order only the quiet moves, after the
 * captures, promotions and killers (quiet_only = 1).  The other moves keep
 * the hand-written order.  Default: top 12, quiet_only 1 (the setting that
 * visits fewer nodes than the hand-written ordering). */
int zeta_search_set_learned_order(int top, int quiet_only);
/* Workers that finish their own position help unfinished ones, up to this
 * many workers per position (0, the default: no helping). */
int zeta_search_set_helpers(int max_workers_per_position);
/* Launch form of the search kernels: 0 automatic (the default), 1 dense --
 * 32 workers per warp, one per thread --, 2 sparse -- one worker per warp,
 * on lane 0, the other lanes exit at once -- or 3 warp-cooperative (pure
 * search only) -- one worker per warp whose lane 0 walks the tree and
 * whose 32 lanes score the children of every node with one ply left.
 * Automatic takes, when every worker of the launch can have a resident
 * warp of its own, the warp-cooperative form for the pure search and the
 * sparse form for the full engine, else the dense form; the full engine
 * treats 3 as automatic.  Root scores do not depend on the form; speed
 * and node counts do.  No counterpart in the reference (one OpenCL work
 * group per worker, zeta.cl:852). */
int zeta_search_set_launch_form(int form);
/* Full engine with more than one worker and no TT2 (lazy SMP, whose
 * helpers randomise their move order, zeta.cl:1980-2001): with every = k
 * >= 2, helpers k-1, 2k-1, ... search one ply deeper than the launch's
 * depth.  They never end the search -- the result is that of a worker at
 * the launch's depth -- and their table entries serve the next
 * iterative-deepening step.  0 (the default) keeps every worker at the
 * launch's depth, as the reference does.  Worker 0, and so a one-worker
 * search, is never affected.  No counterpart in the reference. */
int zeta_engine_set_helper_depth(int every);
/* zero the transposition tables (as a new game does, src/xboard.c:159-199) */
int zeta_tt_clear(void);
/* device time of the last search kernel, ms */
int zeta_search_last_ms(float *kernel_ms);
/* Transposition-table operations of the last batched pure search, counted
 * on the device: probes (one per interior node entered and per depth-1
 * child looked up) and stores (one per finished node).  Each touches one
 * 16-byte entry in one 32-byte DRAM sector, so 32 B x (probes + stores)
 * is the table's traffic (the reference's per-node TT1 load and store,
 * zeta.cl:1623 and 1894-1913). */
int zeta_search_last_table_ops(uint64_t *probes, uint64_t *stores);

/* ------------------------------------------------------------------ */
/* Full-engine search: the reference's alphabeta_gpu (zeta.cl:852-2511)
 * with its heuristics -- quiescence with stand pat, check and promotion
 * extensions, null move (R=2), late move reductions (R=1) with re-search,
 * internal iterative deepening, TT / IID / killer / counter-move ordering,
 * repetition, fifty-move and bare-kings draws, TT1 with the reference's
 * replacement and aging, ABDADA TT2 locks between workers, PV from TT1.
 * One worker searches exactly the reference's tree (same score, PV and
 * node count); more workers share the tables as the reference's
 * work-groups do.  TT1 / TT2 (zeta_init), killer and counter moves persist
 * between calls until zeta_tt_clear, as the reference's device buffers do.
 *
 * One launch: cl_run_alphabeta + cl_read_memory (src/clrun.c:675-974,
 * 1150-1266), depth 0..63; depth 0 is the reference host's start-up
 * warm-up (src/zeta.c:695), a quiescence search of the root as the
 * reference kernel runs it.  hash_history: MAXGAMEPLY (1024) hashes of the game, entry
 * ply_init = this position (NULL: the root hash only); max_nodes stops the
 * search when worker 0 has made more moves (the reference's COUNTERS[1]
 * test).  pv: PV[0] score, PV[1..63] moves, zero when the search was
 * stopped; counters: workers x 64, slot 1 nodes, 3 TT-move hits, 4
 * TT-score hits, 5 IID-move hits (src/search.c:111-117). */
int zeta_engine_search(const uint64_t board[7], int stm, int depth, int ply_init, const uint64_t *hash_history,
                       uint64_t max_nodes, int workers, uint32_t pv[64], uint64_t *counters);
/* n positions in one launch, `workers` each; each position searches with a
 * power-of-two slice (1/n) of TT1 and TT2, ply_init 0.  Outputs per
 * position: score, best move (0 if stopped), nodes summed over workers,
 * and the PV (n x 64, may be NULL). */
int zeta_engine_batch(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, uint64_t max_nodes,
                      int32_t *scores, uint32_t *bestmoves, uint64_t *nodes, uint32_t *pvs);
/* Iterative deepening 1..depth of n positions (rootsearch,
 * src/search.c:35-223, batched): tables, killer and counter moves start
 * empty and carry over between depths; a position stops deepening on a
 * mate it cannot improve, when it has no move, or when worker 0 exceeded
 * max_nodes in one depth (0 = no budget).  ordering: 0 the reference's
 * move ordering, 1 / 2 the move-ordering network (BF16 / FP8) orders the
 * quiet moves at nodes with >= 3 plies left.  Outputs per position: score
 * and best move of the deepest finished depth, nodes summed over depths
 * and workers, that depth (may be NULL); times in ms (wall, search
 * kernels, network; may be NULL). */
int zeta_engine_id(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, uint64_t max_nodes,
                   int ordering, int32_t *scores, uint32_t *bestmoves, uint64_t *nodes, uint8_t *depth_done,
                   float *ms_total, float *ms_search, float *ms_net);

/* ------------------------------------------------------------------ */
/* The move-ordering network (no counterpart in the reference): 768
 * one-hot inputs -> 512 -> 256 ReLU -> (q_from, q_to); a move scores
 * q_from . E_from[from] + q_to . E_to[to].  Trained with Adam on the
 * tensor-core kernels against best moves of the plain search.
 * Parameters: one flat FP32 vector W1 b1 W2 b2 W3 b3 E_from E_to. */
int zeta_mlp_init(uint64_t seed);
int zeta_mlp_param_count(void);
int zeta_mlp_get_params(float *out);
int zeta_mlp_set_params(const float *in);
/* one batch: mean loss and its gradient (no update) */
int zeta_mlp_grads(const uint64_t *boards, const uint8_t *stm, const uint32_t *targets, int n, float *grads,
                   float *loss);
/* epochs over (board, stm, target move); batch a multiple of 128 */
int zeta_mlp_train(const uint64_t *boards, const uint8_t *stm, const uint32_t *targets, int n, int epochs, int batch,
                   float lr, float *loss_per_epoch, float *acc_per_epoch);
/* scores of every legal move (n x 218, engine generation order) */
int zeta_mlp_scores(const uint64_t *boards, const uint8_t *stm, int n, int fp8, float *scores, uint8_t *nmoves,
                    int32_t *best);

/* Tensor-core matrix product used by the move-ordering network (test and
 * tooling entry; no counterpart in the reference): C[M x N] fp32 =
 * A[M x K] . B[N x K]^T, operands K-major BF16 (fp8 == 0) or FP8 E4M3
 * (fp8 != 0), device buffers, K a multiple of 64 (BF16) or 128 (FP8), N a
 * multiple of 16.  tcgen05.mma with FP32 accumulation in tensor memory. */
int zeta_gemm_tc(const void *d_A, const void *d_B, float *d_C, int M, int N, int K, int fp8, void *stream);
/* Kernel choice of the tensor-core products: 0 (default) for short K (at
 * most 32 K slices of 128 bytes per tile, the network's shapes) the
 * persistent kernel -- one CTA per SM walks the output tiles with two
 * tensor-memory accumulators, so a tile's epilogue overlaps the next
 * tile's MMAs -- else the per-tile kernel (its shared-memory ring sized
 * for 2 CTAs per SM, or 1 for split-K launches such as weight gradients); 1 or 2 the per-tile kernel
 * with its ring sized for 1 or 2 resident CTAs per SM; 3 the persistent
 * kernel (split-K launches keep the per-tile one).  Results do not depend
 * on the choice. */
int zeta_gemm_configure(int ctas_per_sm);

/* ------------------------------------------------------------------ */
/* Seeded synthetic positions generated on the device (the benchmark
 * workloads): position i is a pure function of (seed, i), see
 * zeta_gb300/csrc/positions.cu.  Host buffers: boards n*7, stm n,
 * depth n.  Returns ZETA_ERR_DEVICE if some position found no playout
 * meeting the constraints after 64 attempts (its depth is set to 0). */
int zeta_make_positions(uint64_t seed, int n, int min_plies, int max_plies, int min_pieces, int min_depth,
                        int max_depth, uint64_t *boards, uint8_t *stm, uint8_t *depth);

/* Measured 32-bit integer-ALU throughput of the device in Tops/s (lop3 and
 * shf instructions on every SM): the roofline denominator of the perft and
 * search kernels. */
int zeta_int_peak(double *tops);

/* ------------------------------------------------------------------ */
/* Move generation on the device (test and tooling entry): legal moves of
 * n positions, max 256 each, in the reference packing; counts[i] moves
 * for board i.  flags bit 0 keeps captures only; bits 1-2 pick the device
 * generator: 0 the perft generator, 1 the search kernels' (one thread per
 * position), 2 the warp-cooperative search's (one warp per position; the
 * same list as 1, in the same order).  All give the same set; the order
 * within a list differs between 0 and the others.  Bit 3 (perft generator
 * only) adds the rook, bishop and knight promotions after each queen
 * promotion.  Host buffers. */
int zeta_genmoves_batch(const uint64_t *boards, const uint8_t *stm, int n, int flags, uint32_t *moves,
                        int32_t *counts);
/* Static evaluation on the device (test and tooling entry): the reference
 * evaluation of zeta.cl:1479-1544 before the side-to-move negation, in
 * centipawns from white's view, of n boards.  Host buffers. */
int zeta_eval_batch(const uint64_t *boards, int n, int32_t *scores);

#ifdef __cplusplus
}
#endif
#endif
