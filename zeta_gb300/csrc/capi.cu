/*
 * capi.cu -- the extern "C" entry points of libzeta_cuda.so (declared in
 * include/zeta_cuda.h) and the process-wide device context.
 */
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "context.cuh"

namespace zeta {

static Context g_ctx;
static char g_err[512] = "no error";

Context &ctx() { return g_ctx; }

int set_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return set_error(ZETA_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static int require_ready() {
  if (!g_ctx.ready) return set_error(ZETA_ERR_STATE, "zeta_init has not been called");
  return ZETA_OK;
}

/* TT sizing of the reference: the largest power of two of entries that
 * fits in the given megabytes (clrun.c:387-397). */
static uint64_t tt_entries(uint64_t mb, uint64_t entry_bytes) {
  if (mb == 0) return 0;
  uint64_t want = (mb << 20) / entry_bytes;
  uint64_t e = 1;
  while ((e << 1) <= want) e <<= 1;
  return e;
}

/* staging buffers for the host-buffer entry points */
static int ensure_stage(int n) {
  Context &c = g_ctx;
  if (n <= c.stage_cap) return ZETA_OK;
  cudaFree(c.d_boards);
  cudaFree(c.d_stm);
  cudaFree(c.d_depth);
  cudaFree(c.d_leaves);
  if (c.h_pinned) cudaFreeHost(c.h_pinned);
  c.d_boards = nullptr;
  c.d_stm = c.d_depth = nullptr;
  c.d_leaves = nullptr;
  c.h_pinned = nullptr;
  c.stage_cap = 0;
  ZCHECK(cudaMalloc(&c.d_boards, (size_t)n * 7 * sizeof(uint64_t)));
  ZCHECK(cudaMalloc(&c.d_stm, (size_t)n));
  ZCHECK(cudaMalloc(&c.d_depth, (size_t)n));
  ZCHECK(cudaMalloc(&c.d_leaves, (size_t)n * sizeof(uint64_t)));
  c.h_pinned_bytes = (size_t)n * (7 * sizeof(uint64_t) + 2 + sizeof(uint64_t));
  ZCHECK(cudaMallocHost(&c.h_pinned, c.h_pinned_bytes));
  c.stage_cap = n;
  return ZETA_OK;
}

}  // namespace zeta

using namespace zeta;

extern "C" {

const char *zeta_last_error(void) { return g_err; }

int zeta_init(int device, uint64_t tt1_mb, uint64_t tt2_mb) {
  Context &c = g_ctx;
  if (c.ready) return set_error(ZETA_ERR_STATE, "zeta_init called twice without zeta_release");
  int count = 0;
  ZCHECK(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return set_error(ZETA_ERR_ARG, "device %d not present (%d devices)", device, count);
  ZCHECK(cudaSetDevice(device));
  cudaDeviceProp prop;
  ZCHECK(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10)
    return set_error(ZETA_ERR_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a", device, prop.major,
                     prop.minor);
  c.device = device;
  c.sms = prop.multiProcessorCount;
  c.cc_major = prop.major;
  c.cc_minor = prop.minor;
  c.hbm = prop.totalGlobalMem;
  ZCHECK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  for (int i = 0; i < 4; i++) ZCHECK(cudaEventCreate(&c.ev[i]));
  for (int i = 0; i < 2; i++) ZCHECK(cudaEventCreateWithFlags(&c.ev_join[i], cudaEventDisableTiming));
  ZCHECK(cudaMalloc(&c.pc, sizeof(PerftCounters)));
  /* transposition tables, zeroed as cl_init_device does from the host
   * zero images (clrun.c:404-443) */
  c.tt1_entries = tt_entries(tt1_mb, 16);
  c.tt2_entries = tt_entries(tt2_mb, 24);
  if (c.tt1_entries) {
    ZCHECK(cudaMalloc(&c.tt1, c.tt1_entries * 16));
    ZCHECK(cudaMemset(c.tt1, 0, c.tt1_entries * 16));
  }
  if (c.tt2_entries) {
    ZCHECK(cudaMalloc(&c.tt2, c.tt2_entries * 24));
    ZCHECK(cudaMemset(c.tt2, 0, c.tt2_entries * 24));
  }
  c.ready = true;
  return ZETA_OK;
}

int zeta_release(void) {
  Context &c = g_ctx;
  if (!c.ready) return ZETA_OK;
  if (c.graph) cudaGraphExecDestroy(c.graph);
  mlp_free();
  engine_free();
  cudaFree(c.lvl[0]);
  cudaFree(c.lvl[1]);
  cudaFree(c.fin);
  cudaFree(c.pc);
  cudaFree(c.cursors);
  cudaFree(c.scratch);
  cudaFree(c.d_boards);
  cudaFree(c.d_stm);
  cudaFree(c.d_depth);
  cudaFree(c.d_leaves);
  if (c.h_pinned) cudaFreeHost(c.h_pinned);
  cudaFree(c.tt1);
  cudaFree(c.tt2);
  cudaFree(c.s_out);
  cudaFree(c.s_done);
  cudaFree(c.s_busy);
  cudaFree(c.s_status);
  cudaFree(c.s_tt);
  cudaFree(c.s_ocache);
  cudaFree(c.s_oreq);
  cudaFree(c.s_noreq);
  for (int i = 0; i < 4; i++)
    if (c.ev[i]) cudaEventDestroy(c.ev[i]);
  for (int i = 0; i < 2; i++)
    if (c.ev_join[i]) cudaEventDestroy(c.ev_join[i]);
  if (c.stream) cudaStreamDestroy(c.stream);
  c = Context();
  return ZETA_OK;
}

int zeta_device_info(int *sm_count, int *cc_major, int *cc_minor, uint64_t *hbm_bytes) {
  int rc = require_ready();
  if (rc) return rc;
  if (sm_count) *sm_count = g_ctx.sms;
  if (cc_major) *cc_major = g_ctx.cc_major;
  if (cc_minor) *cc_minor = g_ctx.cc_minor;
  if (hbm_bytes) *hbm_bytes = g_ctx.hbm;
  return ZETA_OK;
}

int zeta_perft_configure(const zeta_perft_config *cfg) {
  if (!cfg) return set_error(ZETA_ERR_ARG, "null config");
  if (cfg->task_depth < 1 || cfg->task_depth > 4) return set_error(ZETA_ERR_ARG, "task_depth must be 1..4");
  int t = cfg->threads_per_block;
  if (t != 64 && t != 128 && t != 256 && t != 512)
    return set_error(ZETA_ERR_ARG, "threads_per_block must be 64, 128, 256 or 512");
  if (cfg->blocks_per_sm < 0 || cfg->blocks_per_sm > 32) return set_error(ZETA_ERR_ARG, "blocks_per_sm out of range");
  g_ctx.pcfg = *cfg;
  return ZETA_OK;
}

int zeta_perft_get_config(zeta_perft_config *cfg) {
  if (!cfg) return set_error(ZETA_ERR_ARG, "null config");
  *cfg = g_ctx.pcfg;
  return ZETA_OK;
}

int zeta_perft_set_promotions(int all) {
  if (all != 0 && all != 1) return set_error(ZETA_ERR_ARG, "promotions: 0 (queen only) or 1 (all four pieces)");
  g_ctx.perft_allp = all;
  return ZETA_OK;
}

int zeta_perft_get_promotions(void) { return g_ctx.perft_allp; }

int zeta_perft_last_stats(zeta_perft_stats *st) {
  if (!st) return set_error(ZETA_ERR_ARG, "null stats");
  *st = g_ctx.pstats;
  return ZETA_OK;
}

int zeta_perft_batch_device(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n,
                            uint64_t *d_leaves, void *stream) {
  int rc = require_ready();
  if (rc) return rc;
  if (!d_boards || !d_stm || !d_depth || !d_leaves) return set_error(ZETA_ERR_ARG, "null buffer");
  cudaStream_t s = (cudaStream_t)stream;
  rc = perft_launch(d_boards, d_stm, d_depth, n, d_leaves, s);
  if (rc == ZETA_ERR_CAPACITY) rc = perft_launch(d_boards, d_stm, d_depth, n, d_leaves, s);
  return rc;
}

int zeta_perft_batch(const uint64_t *boards, const uint8_t *stm, const uint8_t *depth, int n, uint64_t *leaves) {
  int rc = require_ready();
  if (rc) return rc;
  if (!boards || !stm || !depth || !leaves || n <= 0) return set_error(ZETA_ERR_ARG, "bad batch arguments");
  rc = ensure_stage(n);
  if (rc) return rc;
  Context &c = g_ctx;
  /* pinned staging so the copies are true DMA */
  uint8_t *hp = (uint8_t *)c.h_pinned;
  uint64_t *hb = (uint64_t *)hp;
  uint8_t *hs = hp + (size_t)n * 56, *hd = hs + n;
  memcpy(hb, boards, (size_t)n * 56);
  memcpy(hs, stm, n);
  memcpy(hd, depth, n);
  ZCHECK(cudaMemcpyAsync(c.d_boards, hb, (size_t)n * 56, cudaMemcpyHostToDevice, c.stream));
  ZCHECK(cudaMemcpyAsync(c.d_stm, hs, n, cudaMemcpyHostToDevice, c.stream));
  ZCHECK(cudaMemcpyAsync(c.d_depth, hd, n, cudaMemcpyHostToDevice, c.stream));
  rc = perft_launch(c.d_boards, c.d_stm, c.d_depth, n, c.d_leaves, c.stream);
  if (rc == ZETA_ERR_CAPACITY) rc = perft_launch(c.d_boards, c.d_stm, c.d_depth, n, c.d_leaves, c.stream);
  if (rc) return rc;
  ZCHECK(cudaMemcpyAsync(leaves, c.d_leaves, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToHost, c.stream));
  ZCHECK(cudaStreamSynchronize(c.stream));
  return ZETA_OK;
}

int zeta_perft(const uint64_t board[7], int stm, int depth, uint64_t *leaves) {
  if (!board || !leaves) return set_error(ZETA_ERR_ARG, "null pointer");
  if (depth < 0 || depth > kMaxDepth) return set_error(ZETA_ERR_ARG, "depth %d outside 0..%d", depth, kMaxDepth);
  uint8_t s = (uint8_t)(stm & 1), d = (uint8_t)depth;
  return zeta_perft_batch(board, &s, &d, 1, leaves);
}

int zeta_make_positions(uint64_t seed, int n, int min_plies, int max_plies, int min_pieces, int min_depth,
                        int max_depth, uint64_t *boards, uint8_t *stm, uint8_t *depth) {
  int rc = require_ready();
  if (rc) return rc;
  if (!boards || !stm || !depth || n <= 0 || min_plies < 0 || max_plies < min_plies || min_depth < 0 ||
      max_depth < min_depth || max_depth > kMaxDepth)
    return set_error(ZETA_ERR_ARG, "bad position-generator arguments");
  Context &c = g_ctx;
  uint64_t *db = nullptr;
  uint8_t *ds = nullptr, *dd = nullptr;
  uint32_t *df = nullptr, fails = 0;
  cudaError_t e = cudaMalloc(&db, (size_t)n * 56);
  if (e == cudaSuccess) e = cudaMalloc(&ds, n);
  if (e == cudaSuccess) e = cudaMalloc(&dd, n);
  if (e == cudaSuccess) e = cudaMalloc(&df, 4);
  if (e == cudaSuccess)
    rc = positions_launch(seed, n, min_plies, max_plies, min_pieces, min_depth, max_depth, db, ds, dd, df, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpyAsync(boards, db, (size_t)n * 56, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpyAsync(stm, ds, n, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpyAsync(depth, dd, n, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpyAsync(&fails, df, 4, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  cudaFree(db);
  cudaFree(ds);
  cudaFree(dd);
  cudaFree(df);
  if (e != cudaSuccess) return cuda_fail(e, "zeta_make_positions");
  if (rc) return rc;
  if (fails) return set_error(ZETA_ERR_DEVICE, "%u positions found no playout meeting the constraints", fails);
  return ZETA_OK;
}

int zeta_int_peak(double *tops) {
  int rc = require_ready();
  if (rc) return rc;
  if (!tops) return set_error(ZETA_ERR_ARG, "null pointer");
  return int_peak(tops);
}

int zeta_search_batch_device(const uint64_t *d_boards, const uint8_t *d_stm, int n, int depth, int workers,
                             int32_t *d_scores, uint32_t *d_bestmoves, uint64_t *d_nodes, void *stream) {
  int rc = require_ready();
  if (rc) return rc;
  if (!d_boards || !d_stm) return set_error(ZETA_ERR_ARG, "null buffer");
  cudaStream_t s = stream ? (cudaStream_t)stream : g_ctx.stream;
  return search_pure_launch(d_boards, d_stm, n, depth, workers, d_scores, d_bestmoves, (unsigned long long *)d_nodes,
                            s);
}

int zeta_search_batch(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, int32_t *scores,
                      uint32_t *bestmoves, uint64_t *nodes) {
  int rc = require_ready();
  if (rc) return rc;
  if (!boards || !stm || n <= 0) return set_error(ZETA_ERR_ARG, "bad batch arguments");
  Context &c = g_ctx;
  uint64_t *db = nullptr, *dn = nullptr;
  uint8_t *ds = nullptr;
  int32_t *dsc = nullptr;
  uint32_t *dm = nullptr;
  cudaError_t e = cudaMalloc(&db, (size_t)n * 56);
  if (e == cudaSuccess) e = cudaMalloc(&ds, n);
  if (e == cudaSuccess) e = cudaMalloc(&dsc, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dm, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dn, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, boards, (size_t)n * 56, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ds, stm, n, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) rc = search_pure_launch(db, ds, n, depth, workers, dsc, dm, (unsigned long long *)dn, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK && scores) e = cudaMemcpy(scores, dsc, (size_t)n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rc == ZETA_OK && bestmoves) e = cudaMemcpy(bestmoves, dm, (size_t)n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rc == ZETA_OK && nodes) e = cudaMemcpy(nodes, dn, (size_t)n * 8, cudaMemcpyDeviceToHost);
  cudaFree(db);
  cudaFree(ds);
  cudaFree(dsc);
  cudaFree(dm);
  cudaFree(dn);
  if (e != cudaSuccess) return cuda_fail(e, "zeta_search_batch");
  return rc;
}

/* One position, one launch (cl_run_alphabeta, src/clrun.c:675-974): the
 * batched search with `workers` ABDADA workers on the single position.
 * pv[0] = score, pv[1] = best move (the rest 0); counters[1] = nodes,
 * counters[4] = transposition-table score hits (src/search.c:114-121
 * reads these slots). */
int zeta_search(const uint64_t board[7], int stm, int depth, int ply_init, const uint64_t *hash_history,
                uint64_t max_nodes, uint32_t pv[64], uint64_t counters[64]) {
  (void)ply_init;
  (void)hash_history;
  (void)max_nodes;
  int rc = require_ready();
  if (rc) return rc;
  if (!board || depth < 1) return set_error(ZETA_ERR_ARG, "bad search arguments");
  uint8_t s = (uint8_t)(stm & 1);
  int32_t score = 0;
  uint32_t move = 0;
  uint64_t nodes = 0;
  rc = zeta_search_batch(board, &s, 1, depth, 64, &score, &move, &nodes);
  if (rc) return rc;
  if (pv) {
    memset(pv, 0, 64 * sizeof(uint32_t));
    pv[0] = (uint32_t)score;
    pv[1] = move;
  }
  if (counters) {
    memset(counters, 0, 64 * sizeof(uint64_t));
    counters[1] = nodes;
  }
  return ZETA_OK;
}

int zeta_search_id(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, int ordering,
                   int32_t *scores, uint32_t *bestmoves, uint64_t *nodes, float *ms_total, float *ms_search,
                   float *ms_net) {
  int rc = require_ready();
  if (rc) return rc;
  if (!boards || !stm || n <= 0 || depth < 1 || workers < 1 || ordering < 0 || ordering > 2)
    return set_error(ZETA_ERR_ARG, "bad search arguments");
  return search_id(boards, stm, n, depth, workers, ordering, scores, bestmoves, nodes, ms_total, ms_search, ms_net);
}

int zeta_search_set_learned_order(int top, int quiet_only) {
  if (top < 1 || top > kOrderTop) return set_error(ZETA_ERR_ARG, "learned top must be 1..%d", kOrderTop);
  g_ctx.s_learned_top = top;
  g_ctx.s_learned_quiet = quiet_only ? 1 : 0;
  return ZETA_OK;
}

int zeta_search_set_helpers(int max_workers_per_position) {
  if (max_workers_per_position < 0) return set_error(ZETA_ERR_ARG, "negative helper cap");
  g_ctx.s_helpers_cap = max_workers_per_position;
  return ZETA_OK;
}

int zeta_engine_set_helper_depth(int every) {
  if (every < 0 || every == 1) return set_error(ZETA_ERR_ARG, "helper depth: 0 (off) or every k-th helper, k >= 2");
  g_ctx.e_deep_every = every;
  return ZETA_OK;
}

int zeta_search_set_launch_form(int form) {
  if (form < 0 || form > 3)
    return set_error(ZETA_ERR_ARG, "launch form must be 0 (auto), 1 (dense), 2 (sparse) or 3 (warp)");
  g_ctx.s_launch_form = form;
  return ZETA_OK;
}

int zeta_tt_clear(void) {
  int rc = require_ready();
  if (rc) return rc;
  rc = search_tt_clear(g_ctx.stream);
  if (rc) return rc;
  rc = engine_clear(g_ctx.stream);
  if (rc) return rc;
  ZCHECK(cudaStreamSynchronize(g_ctx.stream));
  return ZETA_OK;
}

int zeta_search_last_table_ops(uint64_t *probes, uint64_t *stores) {
  if (!probes || !stores) return set_error(ZETA_ERR_ARG, "null pointer");
  *probes = g_ctx.s_probes;
  *stores = g_ctx.s_stores;
  return ZETA_OK;
}

int zeta_search_last_ms(float *kernel_ms) {
  if (!kernel_ms) return set_error(ZETA_ERR_ARG, "null pointer");
  *kernel_ms = g_ctx.sstats.kernel_ms;
  return ZETA_OK;
}

int zeta_eval_batch(const uint64_t *boards, int n, int32_t *scores) {
  int rc = require_ready();
  if (rc) return rc;
  if (!boards || !scores || n <= 0) return set_error(ZETA_ERR_ARG, "bad arguments");
  uint64_t *db = nullptr;
  int32_t *dsc = nullptr;
  Context &c = g_ctx;
  cudaError_t e = cudaMalloc(&db, (size_t)n * 56);
  if (e == cudaSuccess) e = cudaMalloc(&dsc, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, boards, (size_t)n * 56, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) rc = eval_launch(db, n, dsc, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpy(scores, dsc, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaFree(db);
  cudaFree(dsc);
  if (e != cudaSuccess) return cuda_fail(e, "zeta_eval_batch");
  return rc;
}

int zeta_genmoves_batch(const uint64_t *boards, const uint8_t *stm, int n, int flags, uint32_t *moves,
                        int32_t *counts) {
  int rc = require_ready();
  if (rc) return rc;
  if (!boards || !stm || !moves || !counts || n <= 0) return set_error(ZETA_ERR_ARG, "bad arguments");
  uint64_t *db = nullptr;
  uint8_t *ds = nullptr;
  uint32_t *dm = nullptr;
  int32_t *dc = nullptr;
  Context &c = g_ctx;
  cudaError_t e = cudaMalloc(&db, (size_t)n * 56);
  if (e == cudaSuccess) e = cudaMalloc(&ds, n);
  if (e == cudaSuccess) e = cudaMalloc(&dm, (size_t)n * 256 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dc, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, boards, (size_t)n * 56, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ds, stm, n, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) rc = genmoves_launch(db, ds, n, flags, dm, dc, c.stream);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpy(moves, dm, (size_t)n * 256 * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rc == ZETA_OK) e = cudaMemcpy(counts, dc, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaFree(db);
  cudaFree(ds);
  cudaFree(dm);
  cudaFree(dc);
  if (e != cudaSuccess) return cuda_fail(e, "zeta_genmoves_batch");
  return rc;
}

}  // extern "C"
