/*
 * engine.cu -- launch and C ABI of the full-engine search (the worker
 * itself is in engine_core.cuh).
 */
#include <cstdio>
#include <cstring>
#include <vector>

#include "engine_core.cuh"

namespace zeta {

namespace {

/* One worker per thread (dense: 32 workers of different trees share a
 * warp, the most workers resident) or one worker per warp (sparse: lane 0
 * of each warp works alone, so a worker never waits for the other paths
 * of its warp; used when all workers fit on the GPU at once, as in a
 * single-position search). */
template <int TPB>
__global__ void __launch_bounds__(TPB) k_engine(EngineArgs a, int sparse) {
  __shared__ EvalTables sT;
  for (int i = threadIdx.x; i < (int)(sizeof(EvalTables) / 4); i += TPB)
    ((uint32_t *)&sT)[i] = ((const uint32_t *)&kEvalDev)[i];
  __syncthreads();
  long long t = (long long)blockIdx.x * TPB + threadIdx.x;
  if (sparse) {
    if (threadIdx.x & 31) return;
    t >>= 5;
  }
  if (t >= (long long)a.N * a.W) return;
  engine_worker(a, t, sT);
}

constexpr int kEngineTPB = 128;

/* Device state of the full engine: per-worker frames, move lists, game
 * history, killer and counter moves (kept between calls, as the
 * reference keeps its Killer / Counter buffers until the next
 * cl_init_device), and the launch's outputs. */
struct EngineState {
  int cap = 0;      /* workers allocated (N * W) */
  int n_cap = 0;    /* positions allocated */
  int last_n = -1, last_w = -1;
  EFrame *frames = nullptr;
  Move *moves = nullptr;
  u64 *hist = nullptr;
  Move *killers = nullptr;
  Move *cmoves = nullptr;
  unsigned long long *cnt = nullptr;
  uint32_t *finito = nullptr;
  uint32_t *pv = nullptr;
  uint32_t *status = nullptr;
  uint64_t *boards = nullptr;
  uint8_t *stm = nullptr;
  uint8_t *active = nullptr;
  int *ply = nullptr;
  u64 *hist_in = nullptr;
  bool hist_in_alloc = false;
};

EngineState g_eng;

int engine_reserve(int n, int w) {
  Context &c = ctx();
  EngineState &e = g_eng;
  const long long total = (long long)n * w;
  if (total > e.cap) {
    cudaFree(e.frames);
    cudaFree(e.moves);
    cudaFree(e.hist);
    cudaFree(e.killers);
    cudaFree(e.cmoves);
    cudaFree(e.cnt);
    e.frames = nullptr;
    e.cap = 0;
    ZCHECK(cudaMalloc(&e.frames, total * kEFrames * sizeof(EFrame)));
    ZCHECK(cudaMalloc(&e.moves, total * kEFrames * kEMoves * sizeof(Move)));
    ZCHECK(cudaMalloc(&e.hist, total * kGamePly * sizeof(u64)));
    ZCHECK(cudaMalloc(&e.killers, total * kEPly * sizeof(Move)));
    ZCHECK(cudaMalloc(&e.cmoves, total * 4096 * sizeof(Move)));
    ZCHECK(cudaMalloc(&e.cnt, total * 4 * sizeof(unsigned long long)));
    e.cap = (int)total;
    e.last_n = -1;
  }
  if (n > e.n_cap) {
    cudaFree(e.finito);
    cudaFree(e.pv);
    cudaFree(e.boards);
    cudaFree(e.stm);
    cudaFree(e.active);
    cudaFree(e.ply);
    ZCHECK(cudaMalloc(&e.finito, n * sizeof(uint32_t)));
    ZCHECK(cudaMalloc(&e.pv, (size_t)n * kEPly * sizeof(uint32_t)));
    ZCHECK(cudaMalloc(&e.boards, (size_t)n * 7 * sizeof(uint64_t)));
    ZCHECK(cudaMalloc(&e.stm, n));
    ZCHECK(cudaMalloc(&e.active, n));
    ZCHECK(cudaMalloc(&e.ply, n * sizeof(int)));
    e.n_cap = n;
  }
  if (!e.status) ZCHECK(cudaMalloc(&e.status, sizeof(uint32_t)));
  if (n != e.last_n || w != e.last_w) {
    /* a new batch shape: killer and counter moves start empty */
    ZCHECK(cudaMemsetAsync(e.killers, 0, total * kEPly * sizeof(Move), c.stream));
    ZCHECK(cudaMemsetAsync(e.cmoves, 0, total * 4096 * sizeof(Move), c.stream));
    e.last_n = n;
    e.last_w = w;
  }
  return ZETA_OK;
}

u64 pow2_floor(u64 x) {
  u64 p = 1;
  while (p <= x / 2) p <<= 1;
  return x ? p : 0;
}

}  // namespace

/* tables and killers back to zero (a new game) */
int engine_clear(cudaStream_t s) {
  Context &c = ctx();
  EngineState &e = g_eng;
  if (c.tt1) ZCHECK(cudaMemsetAsync(c.tt1, 0, c.tt1_entries * 16, s));
  if (c.tt2) ZCHECK(cudaMemsetAsync(c.tt2, 0, c.tt2_entries * 24, s));
  if (e.killers && e.cap) {
    ZCHECK(cudaMemsetAsync(e.killers, 0, (size_t)e.cap * kEPly * sizeof(Move), s));
    ZCHECK(cudaMemsetAsync(e.cmoves, 0, (size_t)e.cap * 4096 * sizeof(Move), s));
  }
  return ZETA_OK;
}

void engine_free() {
  EngineState &e = g_eng;
  cudaFree(e.frames);
  cudaFree(e.moves);
  cudaFree(e.hist);
  cudaFree(e.killers);
  cudaFree(e.cmoves);
  cudaFree(e.cnt);
  cudaFree(e.finito);
  cudaFree(e.pv);
  cudaFree(e.status);
  cudaFree(e.boards);
  cudaFree(e.stm);
  cudaFree(e.active);
  cudaFree(e.ply);
  cudaFree(e.hist_in);
  e = EngineState();
}

/* One fixed-depth launch over n positions already staged in g_eng
 * (boards, stm, ply, active, optional history).  Each position gets a
 * power-of-two slice of TT1 / TT2. */
int engine_launch(int n, int w, int depth, uint64_t max_nodes, bool with_hist, bool with_active, float *kernel_ms,
                  bool learned = false) {
  Context &c = ctx();
  EngineState &e = g_eng;
  if (c.tt_owner != 2) {
    /* the pure search keeps a different entry format in the same memory */
    int rc = engine_clear(c.stream);
    if (rc) return rc;
    c.tt_owner = 2;
  }
  EngineArgs a{};
  a.boards = e.boards;
  a.stm = e.stm;
  a.hist_in = with_hist ? e.hist_in : nullptr;
  a.ply_init = e.ply;
  a.active = with_active ? e.active : nullptr;
  a.N = n;
  a.W = w;
  a.depth = depth;
  a.max_nodes = max_nodes;
  const unsigned long long cap = 1ull << 40;
  a.iter_budget = max_nodes > (cap >> 3) ? cap : 4 * max_nodes + (1u << 20);
  a.tt1 = (TT1E *)c.tt1;
  a.tt1_slice = c.tt1 ? pow2_floor(c.tt1_entries / (u64)n) : 0;
  a.tt2 = (TT2E *)c.tt2;
  a.tt2_slice = c.tt2 ? pow2_floor(c.tt2_entries / (u64)n) : 0;
  a.frames = e.frames;
  a.moves = e.moves;
  a.hist = e.hist;
  a.killers = e.killers;
  a.cmoves = e.cmoves;
  a.cnt = e.cnt;
  a.finito = e.finito;
  a.pv = e.pv;
  a.status = e.status;
  a.deep_every = c.e_deep_every;
  if (learned) {
    a.ocache = (OrderEntry *)c.s_ocache;
    a.ocache_mask = c.s_ocache_entries - 1;
    a.oreq = (OrderRequest *)c.s_oreq;
    a.noreq = c.s_noreq;
    a.oreq_cap = c.s_oreq_cap;
    a.learned_top = c.s_learned_top;
  }
  ZCHECK(cudaMemsetAsync(e.finito, 0, n * sizeof(uint32_t), c.stream));
  ZCHECK(cudaMemsetAsync(e.pv, 0, (size_t)n * kEPly * sizeof(uint32_t), c.stream));
  ZCHECK(cudaMemsetAsync(e.status, 0, sizeof(uint32_t), c.stream));
  const long long total = (long long)n * w;
  /* sparse when every worker can have a resident warp of its own; the
   * sparse form launches one-warp blocks, so that the block scheduler
   * spreads the workers over all SMs instead of packing four per SM */
  static int resident_warps = 0;
  if (!resident_warps) {
    int per_sm = 0;
    ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_engine<32>, 32, 0));
    resident_warps = (per_sm > 0 ? per_sm : 1) * c.sms;
  }
  /* form 3 (warp-cooperative) is a pure-search form: the engine takes its automatic choice */
  const int form = c.s_launch_form == 1 || c.s_launch_form == 2 ? c.s_launch_form : 0;
  const int sparse = form ? (form == 2 ? 1 : 0) : (total <= (long long)resident_warps ? 1 : 0);
  ZCHECK(cudaEventRecord(c.ev[0], c.stream));
  if (sparse)
    k_engine<32><<<(unsigned)total, 32, 0, c.stream>>>(a, 1);
  else
    k_engine<kEngineTPB><<<(unsigned)((total + kEngineTPB - 1) / kEngineTPB), kEngineTPB, 0, c.stream>>>(a, 0);
  ZCHECK(cudaGetLastError());
  ZCHECK(cudaEventRecord(c.ev[1], c.stream));
  ZCHECK(cudaStreamSynchronize(c.stream));
  if (kernel_ms) ZCHECK(cudaEventElapsedTime(kernel_ms, c.ev[0], c.ev[1]));
  uint32_t st = 0;
  ZCHECK(cudaMemcpy(&st, e.status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st & EST_BUDGET) return set_error(ZETA_ERR_BUDGET, "engine: a worker ran out of loop iterations");
  return ZETA_OK;
}

int engine_stage(const uint64_t *boards, const uint8_t *stm, int n, int w, const int *ply_init,
                 const uint64_t *hist, int hist_rows) {
  Context &c = ctx();
  EngineState &e = g_eng;
  int rc = engine_reserve(n, w);
  if (rc) return rc;
  ZCHECK(cudaMemcpyAsync(e.boards, boards, (size_t)n * 7 * sizeof(uint64_t), cudaMemcpyHostToDevice, c.stream));
  ZCHECK(cudaMemcpyAsync(e.stm, stm, n, cudaMemcpyHostToDevice, c.stream));
  std::vector<int> ply(n, 0);
  if (ply_init)
    for (int i = 0; i < n; i++) ply[i] = ply_init[i];
  ZCHECK(cudaMemcpyAsync(e.ply, ply.data(), n * sizeof(int), cudaMemcpyHostToDevice, c.stream));
  if (hist) {
    cudaFree(e.hist_in);
    e.hist_in = nullptr;
    ZCHECK(cudaMalloc(&e.hist_in, (size_t)n * kGamePly * sizeof(u64)));
    for (int i = 0; i < n; i++)
      ZCHECK(cudaMemcpyAsync(e.hist_in + (size_t)i * kGamePly, hist + (size_t)(hist_rows > 1 ? i : 0) * kGamePly,
                             kGamePly * sizeof(u64), cudaMemcpyHostToDevice, c.stream));
  }
  ZCHECK(cudaStreamSynchronize(c.stream));
  return ZETA_OK;
}

EngineState &engine_state() { return g_eng; }

}  // namespace zeta

using namespace zeta;

extern "C" int zeta_engine_search(const uint64_t board[7], int stm, int depth, int ply_init,
                                  const uint64_t *hash_history, uint64_t max_nodes, int workers, uint32_t pv[64],
                                  uint64_t *counters) {
  Context &c = ctx();
  if (!c.ready) return set_error(ZETA_ERR_STATE, "zeta_init has not been called");
  if (!board || !pv || !counters) return set_error(ZETA_ERR_ARG, "null pointer");
  /* depth 0 is the reference host's start-up warm-up (src/zeta.c:695): a
   * quiescence search of the root, as the reference kernel runs it */
  if (depth < 0 || depth >= kEPly) return set_error(ZETA_ERR_ARG, "depth %d out of range 0..%d", depth, kEPly - 1);
  if (workers < 1 || workers > 65536) return set_error(ZETA_ERR_ARG, "workers %d out of range", workers);
  if (ply_init < 0 || ply_init >= kGamePly) return set_error(ZETA_ERR_ARG, "ply_init %d out of range", ply_init);
  uint8_t s = (uint8_t)(stm & 1);
  int rc = engine_stage(board, &s, 1, workers, &ply_init, hash_history, 1);
  if (rc) return rc;
  rc = engine_launch(1, workers, depth, max_nodes, hash_history != nullptr, false, &c.sstats.kernel_ms);
  if (rc) return rc;
  EngineState &e = engine_state();
  ZCHECK(cudaMemcpy(pv, e.pv, kEPly * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> cnt((size_t)workers * 4);
  ZCHECK(cudaMemcpy(cnt.data(), e.cnt, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  memset(counters, 0, (size_t)workers * 64 * sizeof(uint64_t));
  for (int w = 0; w < workers; w++) {
    counters[w * 64 + 1] = cnt[w * 4 + 0]; /* nodes */
    counters[w * 64 + 3] = cnt[w * 4 + 1]; /* TT move hits */
    counters[w * 64 + 4] = cnt[w * 4 + 2]; /* TT score hits */
    counters[w * 64 + 5] = cnt[w * 4 + 3]; /* IID move hits */
  }
  return ZETA_OK;
}

extern "C" int zeta_engine_batch(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers,
                                 uint64_t max_nodes, int32_t *scores, uint32_t *bestmoves, uint64_t *nodes,
                                 uint32_t *pvs) {
  Context &c = ctx();
  if (!c.ready) return set_error(ZETA_ERR_STATE, "zeta_init has not been called");
  if (!boards || !stm || !scores || !bestmoves || !nodes) return set_error(ZETA_ERR_ARG, "null pointer");
  if (n < 1 || depth < 1 || depth >= kEPly || workers < 1 || (long long)n * workers > (1ll << 24))
    return set_error(ZETA_ERR_ARG, "engine batch: n %d depth %d workers %d out of range", n, depth, workers);
  int rc = engine_stage(boards, stm, n, workers, nullptr, nullptr, 0);
  if (rc) return rc;
  rc = engine_launch(n, workers, depth, max_nodes, false, false, &c.sstats.kernel_ms);
  if (rc) return rc;
  EngineState &e = engine_state();
  std::vector<uint32_t> pv((size_t)n * kEPly);
  ZCHECK(cudaMemcpy(pv.data(), e.pv, pv.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> cnt((size_t)n * workers * 4);
  ZCHECK(cudaMemcpy(cnt.data(), e.cnt, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; i++) {
    scores[i] = (int32_t)pv[(size_t)i * kEPly];
    bestmoves[i] = pv[(size_t)i * kEPly + 1];
    uint64_t s = 0;
    for (int w = 0; w < workers; w++) s += cnt[((size_t)w * n + i) * 4];
    nodes[i] = s;
  }
  if (pvs) memcpy(pvs, pv.data(), pv.size() * sizeof(uint32_t));
  return ZETA_OK;
}

/* Iterative deepening 1..depth over a batch (rootsearch,
 * src/search.c:35-223, for n positions at once): tables, killer and
 * counter moves start empty and carry over between depths; a position
 * stops deepening on a mate-in-n it cannot improve, on a missing move or
 * when worker 0 ran out of its node budget.  ordering 1 / 2: the
 * move-ordering network (BF16 / FP8) orders the quiet moves of nodes with
 * >= 3 plies left, from requests logged in the previous depth. */
extern "C" int zeta_engine_id(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers,
                              uint64_t max_nodes, int ordering, int32_t *scores, uint32_t *bestmoves, uint64_t *nodes,
                              uint8_t *depth_done, float *ms_total, float *ms_search, float *ms_net) {
  Context &c = ctx();
  if (!c.ready) return set_error(ZETA_ERR_STATE, "zeta_init has not been called");
  if (!boards || !stm || !scores || !bestmoves || !nodes) return set_error(ZETA_ERR_ARG, "null pointer");
  if (n < 1 || depth < 1 || depth >= kEPly || workers < 1 || (long long)n * workers > (1ll << 24) || ordering < 0 ||
      ordering > 2)
    return set_error(ZETA_ERR_ARG, "engine id: n %d depth %d workers %d ordering %d out of range", n, depth, workers,
                     ordering);
  const bool learned = ordering > 0;
  if (learned && !mlp_ready_for_search())
    return set_error(ZETA_ERR_STATE, "learned ordering needs zeta_mlp_init (and training or parameters)");
  int rc = engine_stage(boards, stm, n, workers, nullptr, nullptr, 0);
  if (rc) return rc;
  rc = engine_clear(c.stream);
  if (rc) return rc;
  c.tt_owner = 2;
  if (learned) {
    rc = learn_buffers();
    if (rc) return rc;
    ZCHECK(cudaMemsetAsync(c.s_ocache, 0, c.s_ocache_entries * sizeof(OrderEntry), c.stream));
    ZCHECK(cudaMemsetAsync(c.s_noreq, 0, 4, c.stream));
  }
  EngineState &e = engine_state();
  std::vector<uint8_t> active(n, 1);
  std::vector<uint32_t> pv((size_t)n * kEPly);
  std::vector<unsigned long long> cnt((size_t)n * workers * 4);
  for (int i = 0; i < n; i++) {
    scores[i] = 0;
    bestmoves[i] = 0;
    nodes[i] = 0;
    if (depth_done) depth_done[i] = 0;
  }
  float t_search = 0.f, t_net = 0.f;
  const uint64_t budget = max_nodes ? max_nodes : ~0ULL;
  ZCHECK(cudaEventRecord(c.ev[2], c.stream));
  for (int d = 1; d <= depth; d++) {
    int live = 0;
    for (int i = 0; i < n; i++) live += active[i];
    if (!live) break;
    ZCHECK(cudaMemcpyAsync(e.active, active.data(), n, cudaMemcpyHostToDevice, c.stream));
    float ms = 0.f;
    rc = engine_launch(n, workers, d, budget, false, true, &ms, learned);
    if (rc) return rc;
    t_search += ms;
    ZCHECK(cudaMemcpy(pv.data(), e.pv, pv.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    ZCHECK(cudaMemcpy(cnt.data(), e.cnt, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) {
      if (!active[i]) continue;
      for (int w = 0; w < workers; w++) nodes[i] += cnt[((size_t)w * n + i) * 4];
      const uint32_t *P = &pv[(size_t)i * kEPly];
      const bool stopped = cnt[(size_t)i * 4] >= budget;
      if (stopped || (P[1] & 0x3FFFFFFFu) == 0) {
        active[i] = 0;
        continue;
      }
      const int sc = (int32_t)P[0];
      bestmoves[i] = P[1];
      scores[i] = is_inf(sc) ? 0 : sc;
      if (depth_done) depth_done[i] = (uint8_t)d;
      if ((sc >= E_MATE && sc < E_INF && d >= E_INF - sc) || (sc <= -E_MATE && sc > -E_INF && d >= E_INF + sc))
        active[i] = 0; /* mate in n found */
    }
    if (learned && d < depth) {
      uint32_t nreq = 0;
      ZCHECK(cudaMemcpy(&nreq, c.s_noreq, 4, cudaMemcpyDeviceToHost));
      if (nreq > c.s_oreq_cap) nreq = c.s_oreq_cap;
      ZCHECK(cudaEventRecord(c.ev[0], c.stream));
      if (nreq)
        rc = mlp_fill_order_cache((const OrderRequest *)c.s_oreq, nreq, (OrderEntry *)c.s_ocache,
                                  c.s_ocache_entries - 1, ordering == 2, c.stream);
      if (rc) return rc;
      ZCHECK(cudaEventRecord(c.ev[1], c.stream));
      ZCHECK(cudaEventSynchronize(c.ev[1]));
      float mm = 0.f;
      ZCHECK(cudaEventElapsedTime(&mm, c.ev[0], c.ev[1]));
      t_net += mm;
      ZCHECK(cudaMemsetAsync(c.s_noreq, 0, 4, c.stream));
    }
  }
  ZCHECK(cudaEventRecord(c.ev[3], c.stream));
  ZCHECK(cudaEventSynchronize(c.ev[3]));
  float tot = 0.f;
  ZCHECK(cudaEventElapsedTime(&tot, c.ev[2], c.ev[3]));
  if (ms_total) *ms_total = tot;
  if (ms_search) *ms_search = t_search;
  if (ms_net) *ms_net = t_net;
  return ZETA_OK;
}
