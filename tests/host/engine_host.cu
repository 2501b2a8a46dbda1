/*
 * engine_host.cu -- the full-engine worker (engine_core.cuh) compiled for
 * the host (nvcc, host code only), one worker, for the CPU parity test
 * against the reference kernel run by refshim.  he_new allocates the
 * tables and per-worker state; he_run searches one position to a depth
 * with the tables, killer and counter moves kept from the previous call,
 * as the reference host does between iterative-deepening depths.
 */
#include <vector>

#include "../../zeta_gb300/csrc/engine_core.cuh"

using namespace zeta;

struct HostEngine {
  std::vector<TT1E> tt1;
  std::vector<TT2E> tt2;
  std::vector<EFrame> frames;
  std::vector<Move> moves, killers, cmoves;
  std::vector<u64> hist, hin;
  std::vector<unsigned long long> cnt;
  std::vector<uint32_t> finito, pv, status;
  std::vector<int> ply;
  std::vector<uint8_t> stm;
  std::vector<uint64_t> board;
  u64 e1, e2;
};

extern "C" void *he_new(uint64_t tt1_entries, uint64_t tt2_entries) {
  HostEngine *h = new HostEngine();
  h->e1 = tt1_entries;
  h->e2 = tt2_entries;
  h->tt1.assign(tt1_entries ? tt1_entries : 1, TT1E{});
  h->tt2.assign(tt2_entries ? tt2_entries : 1, TT2E{});
  h->frames.resize(kEFrames);
  h->moves.resize(kEFrames * kEMoves);
  h->hist.resize(kGamePly);
  h->hin.resize(kGamePly);
  h->killers.assign(kEPly, 0);
  h->cmoves.assign(4096, 0);
  h->cnt.assign(4, 0);
  h->finito.assign(1, 0);
  h->pv.assign(64, 0);
  h->status.assign(1, 0);
  h->ply.assign(1, 0);
  h->stm.assign(1, 0);
  h->board.assign(7, 0);
  return h;
}

extern "C" void he_free(void *hp) { delete (HostEngine *)hp; }

extern "C" void he_run(void *hp, const uint64_t *board, int stm, int depth, int ply_init, const uint64_t *hist,
                       uint64_t max_nodes, uint32_t *pv, uint64_t *counters) {
  HostEngine *h = (HostEngine *)hp;
  for (int i = 0; i < 7; i++) h->board[i] = board[i];
  h->stm[0] = (uint8_t)stm;
  h->ply[0] = ply_init;
  if (hist)
    for (int i = 0; i < kGamePly; i++) h->hin[i] = hist[i];
  std::fill(h->pv.begin(), h->pv.end(), 0u);
  h->finito[0] = 0;
  h->status[0] = 0;
  EngineArgs a{};
  a.boards = h->board.data();
  a.stm = h->stm.data();
  a.hist_in = hist ? h->hin.data() : nullptr;
  a.ply_init = h->ply.data();
  a.active = nullptr;
  a.N = 1;
  a.W = 1;
  a.depth = depth;
  a.max_nodes = max_nodes;
  a.iter_budget = 1ull << 40;
  a.tt1 = h->tt1.data();
  a.tt1_slice = h->e1;
  a.tt2 = h->tt2.data();
  a.tt2_slice = h->e2;
  a.frames = h->frames.data();
  a.moves = h->moves.data();
  a.hist = h->hist.data();
  a.killers = h->killers.data();
  a.cmoves = h->cmoves.data();
  a.cnt = h->cnt.data();
  a.finito = h->finito.data();
  a.pv = h->pv.data();
  a.status = h->status.data();
  engine_worker(a, 0, kEvalHost);
  for (int i = 0; i < 64; i++) pv[i] = h->pv[i];
  for (int i = 0; i < 64; i++) counters[i] = 0;
  counters[1] = h->cnt[0];
  counters[3] = h->cnt[1];
  counters[4] = h->cnt[2];
  counters[5] = h->cnt[3];
}
