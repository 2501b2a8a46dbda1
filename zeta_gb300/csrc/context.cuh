/*
 * context.cuh -- device state of libzeta_cuda.so (internal).
 *
 * One context per process, as the reference keeps one OpenCL context in
 * globals (src/zeta.c:56-139).  It owns the stream, the perft work
 * arena, the transposition tables and the staging buffers of the
 * host-buffer entry points.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zeta_cuda.h"
#include "chess.cuh"

namespace zeta {

/* One subtree of a perft launch: a position, its side to move, its
 * remaining depth and the batch index whose count it adds to. 48 bytes. */
struct __align__(16) Task {
  Pos pos;
  uint32_t root;
  uint8_t stm;
  uint8_t depth;
  uint16_t pad;
};

/* The move-ordering network's ordering of a search node: its 12 best
 * moves as (from | to << 6); 0xFFFF marks an empty slot (all empty: the
 * node was requested and is not scored yet). 32 bytes. */
constexpr int kOrderTop = 12;
struct OrderEntry {
  unsigned long long key;
  uint16_t mv[kOrderTop];
};
/* a search node whose ordering the next kernel step computes */
struct OrderRequest {
  unsigned long long key;
  unsigned long long b[5];
  uint32_t stm, pad;
};

constexpr int kMaxLevels = 12;   /* split levels per launch: depth <= 15 */
constexpr int kMaxDepth = 15;

/* device-side counters of one perft launch */
struct PerftCounters {
  uint32_t level_n[kMaxLevels + 1]; /* nodes per split level */
  uint32_t n_final;                 /* subtree tasks */
  uint32_t status;                  /* ZETA_ERR_* as positive bits, 0 = fine */
  uint32_t pad;
  unsigned long long steals;
  unsigned long long interior;
  unsigned long long counted;
};

struct Context {
  bool ready = false;
  int device = 0;
  int sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t hbm = 0;
  cudaStream_t stream = nullptr;

  /* perft arena */
  Task *lvl[2] = {nullptr, nullptr};
  Task *fin = nullptr;
  uint32_t cap_lvl = 0, cap_fin = 0;
  PerftCounters *pc = nullptr;
  uint32_t *cursors = nullptr;
  int cursors_cap = 0;
  Pos *scratch = nullptr;    /* per-block node buffers of the work-stealing kernel */
  uint64_t scratch_cap = 0;  /* positions */

  /* staging for host-buffer calls */
  uint64_t *d_boards = nullptr;
  uint8_t *d_stm = nullptr, *d_depth = nullptr;
  uint64_t *d_leaves = nullptr;
  int stage_cap = 0;
  void *h_pinned = nullptr;
  size_t h_pinned_bytes = 0;

  /* the autotuner's choice on GB300 (zeta_gb300/perft_tuned.json) */
  zeta_perft_config pcfg{256, 3, 0, 4, 1};
  int perft_allp = 0; /* 1: perft promotes to all four pieces; 0: queen only, the reference's rule */
  zeta_perft_stats pstats{};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev_join[2] = {nullptr, nullptr}; /* ordering with a caller's stream */

  /* cached CUDA graph of the last perft launch sequence */
  cudaGraphExec_t graph = nullptr;
  const void *g_boards = nullptr, *g_stm = nullptr, *g_depth = nullptr, *g_leaves = nullptr;
  int g_n = -1;
  cudaStream_t g_stream = nullptr;
  zeta_perft_config g_cfg{};
  int g_allp = 0;

  /* transposition tables (search) */
  void *mlp = nullptr; /* move-ordering network state (mlp.cu) */
  int tt_owner = 0;    /* entry format held in tt1: 1 pure search, 2 full engine */
  void *tt1 = nullptr, *tt2 = nullptr;
  uint64_t tt1_entries = 0, tt2_entries = 0;

  /* batched search */
  void *s_out = nullptr;      /* per-position results */
  uint32_t *s_done = nullptr; /* early-bird flags */
  int s_cap = 0;
  uint32_t *s_busy = nullptr; /* ABDADA busy table */
  uint64_t s_busy_entries = 0;
  uint32_t *s_status = nullptr;
  unsigned long long s_probes = 0, s_stores = 0; /* table operations of the last batched search */
  int s_helpers_cap = 0;      /* max workers per position once helpers join; 0 = no helpers */
  int s_launch_form = 0;      /* search kernels: 0 auto, 1 dense, 2 sparse, 3 warp (pure search) */
  int e_deep_every = 0;       /* full engine, lazy SMP: every k-th helper one ply deeper (0 = off) */
  int s_learned_top = 12;     /* network moves used by the learned ordering */
  int s_learned_quiet = 1;    /* 1: they order the quiet moves only */
  void *s_ocache = nullptr;   /* learned ordering: OrderEntry cache */
  uint64_t s_ocache_entries = 0;
  void *s_oreq = nullptr;     /* OrderRequest log of the current kernel step */
  uint32_t *s_noreq = nullptr;
  uint32_t s_oreq_cap = 0;
  void *s_tt = nullptr;       /* used when zeta_init made no table */
  uint64_t s_tt_entries = 0;
  struct {
    float kernel_ms = -1.f;
  } sstats;
};

Context &ctx();
int set_error(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define ZCHECK(call)                                   \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

/* perft.cu */
int perft_launch(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n,
                 uint64_t *d_leaves, cudaStream_t stream);
int perft_ensure_arena(uint64_t tasks_cap);
int positions_launch(u64 seed, int n, int min_plies, int max_plies, int min_pieces, int min_depth, int max_depth,
                     uint64_t *d_boards, uint8_t *d_stm, uint8_t *d_depth, uint32_t *d_fail, cudaStream_t s);
int int_peak(double *tops);
/* search.cu */
int search_pure_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int depth, int workers, int32_t *d_scores,
                       uint32_t *d_moves, unsigned long long *d_nodes, cudaStream_t s, int learned = 0);
int search_id(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, int ordering, int32_t *scores,
              uint32_t *moves, uint64_t *nodes, float *ms_total, float *ms_search, float *ms_mlp);
/* mlp.cu: score the logged requests and fill the ordering cache */
int mlp_fill_order_cache(const OrderRequest *req, uint32_t nreq, OrderEntry *cache, uint64_t mask, int fp8,
                         cudaStream_t s);
bool mlp_ready_for_search();
int learn_buffers();
int search_tt_clear(cudaStream_t s);
int eval_launch(const uint64_t *d_boards, int n, int32_t *d_scores, cudaStream_t s);
/* mlp.cu */
void mlp_free();
/* engine.cu: the full-engine search */
int engine_clear(cudaStream_t s);
void engine_free();
int warp_genmoves_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int qs, uint32_t *d_moves,
                         int32_t *d_counts, cudaStream_t s);
int genmoves_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int flags, uint32_t *d_moves,
                    int32_t *d_counts, cudaStream_t stream);

}  // namespace zeta
