/*
 * refshim.cc -- C API over the reference kernels compiled for the host
 * (kernel_perft.cc, kernel_search.cc).  TEST INFRASTRUCTURE ONLY: the
 * bit-exact parity pin for the CUDA kernels and the timed "reference
 * kernels on host cores" baseline.  Buffer shapes follow what clrun.c
 * allocates for one worker (clrun.c:278-511).
 */
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../zeta_oracle.h"
#include "fiber.h"

extern "C" {
void refshim_perft_lane(const unsigned long *board, unsigned long *counters, unsigned long *moves,
                        unsigned long *history, const unsigned long *between,
                        const unsigned long *line, int stm, int depth);
void refshim_search_lane(const unsigned long *board, unsigned long *counters,
                         const unsigned int *rnumbers, unsigned int *pv, unsigned long *moves1,
                         unsigned long *moves2, unsigned long *history,
                         const unsigned long *between, const unsigned long *line, void *tt1,
                         void *tt2, unsigned int *killers, unsigned int *countermoves, int stm,
                         int ply_init, int depth, unsigned long max_nodes,
                         unsigned long tt1_entries, unsigned long tt2_entries,
                         unsigned int *finito);
int refshim_tte_size(void);
int refshim_abdadatte_size(void);
}

namespace {
constexpr int kMaxPly = 64;        /* MAXPLY, zeta.cl / zetaperft.cl */
constexpr int kMaxGamePly = 1024;  /* MAXGAMEPLY */

struct PerftArgs {
  const unsigned long *board;
  unsigned long *counters;
  unsigned long *moves;
  unsigned long *history;
  int stm, depth;
};

void perft_body(void *p) {
  PerftArgs *a = (PerftArgs *)p;
  refshim_perft_lane(a->board, a->counters, a->moves, a->history,
                     (const unsigned long *)zo_inbetween_table(),
                     (const unsigned long *)zo_line_table(), a->stm, a->depth);
}

uint64_t perft_one(const uint64_t board[7], int stm, int depth) {
  std::vector<unsigned long> counters(64, 0), moves(kMaxPly * 64, 0), history(kMaxGamePly, 0);
  PerftArgs a{(const unsigned long *)board, counters.data(), moves.data(), history.data(), stm, depth};
  refshim::run_workgroup(perft_body, &a, 64);
  return counters[1];
}
}  // namespace

extern "C" {

uint64_t ref_perft(const uint64_t board[7], int stm, int depth) {
  zo_inbetween_table();
  return perft_one(board, stm, depth);
}

void ref_perft_batch(const uint64_t *boards, const int *stm, const int *depth, int n, uint64_t *out,
                     int threads) {
  zo_inbetween_table(); /* build shared tables before the threads start */
  std::atomic<int> next(0);
  auto worker = [&]() {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= n) break;
      out[i] = perft_one(boards + 7 * (size_t)i, stm[i], depth[i]);
    }
  };
  if (threads < 1) threads = 1;
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(worker);
  for (auto &t : pool) t.join();
}

/* One position, root moves fanned out over threads; every subtree count
 * comes from the reference kernel. */
uint64_t ref_perft_split(const uint64_t board[7], int stm, int depth, int threads) {
  if (depth <= 1) return ref_perft(board, stm, depth);
  zo_move moves[ZO_MAXMOVES];
  int n = zo_genmoves(board, stm, 0, moves);
  std::vector<uint64_t> kids(7 * (size_t)n), out(n);
  std::vector<int> s(n, !stm), d(n, depth - 1);
  for (int i = 0; i < n; i++) {
    memcpy(&kids[7 * (size_t)i], board, 7 * sizeof(uint64_t));
    zo_play(&kids[7 * (size_t)i], stm, moves[i], 1);
  }
  ref_perft_batch(kids.data(), s.data(), d.data(), n, out.data(), threads);
  uint64_t total = 0;
  for (int i = 0; i < n; i++) total += out[i];
  return total;
}

/* ---------------- search ---------------- */
struct RefSearch {
  uint64_t tt1_entries, tt2_entries;
  int workers;
  std::vector<unsigned char> tt1, tt2;
  std::vector<unsigned int> killers, countermoves;
};

void *ref_search_new(uint64_t tt1_entries, uint64_t tt2_entries, int workers) {
  zo_inbetween_table();
  RefSearch *s = new RefSearch();
  s->tt1_entries = tt1_entries;
  s->tt2_entries = tt2_entries;
  s->workers = workers < 1 ? 1 : workers;
  s->tt1.assign((size_t)(tt1_entries ? tt1_entries : 1) * refshim_tte_size(), 0);
  s->tt2.assign((size_t)(tt2_entries ? tt2_entries : 1) * refshim_abdadatte_size(), 0);
  s->killers.assign((size_t)s->workers * kMaxPly, 0);
  s->countermoves.assign((size_t)s->workers * 64 * 64, 0);
  return s;
}

void ref_search_free(void *h) { delete (RefSearch *)h; }

void ref_search_clear(void *h) {
  RefSearch *s = (RefSearch *)h;
  std::fill(s->tt1.begin(), s->tt1.end(), 0);
  std::fill(s->tt2.begin(), s->tt2.end(), 0);
  std::fill(s->killers.begin(), s->killers.end(), 0);
  std::fill(s->countermoves.begin(), s->countermoves.end(), 0);
}

namespace {
struct SearchLaunch {
  RefSearch *s;
  const uint64_t *board;
  std::vector<unsigned long> *counters;
  const unsigned int *rnumbers;
  unsigned int *pv;
  std::vector<unsigned long> *moves1, *moves2, *history;
  unsigned int *finito;
  int stm, ply_init, depth;
  uint64_t max_nodes;
  int gid;
};

thread_local SearchLaunch *t_launch;

void search_body(void *p) {
  SearchLaunch *L = (SearchLaunch *)p;
  refshim_search_lane((const unsigned long *)L->board, L->counters->data(), L->rnumbers, L->pv,
                      L->moves1->data(), L->moves2->data(), L->history->data(),
                      (const unsigned long *)zo_inbetween_table(),
                      (const unsigned long *)zo_line_table(), L->s->tt1.data(), L->s->tt2.data(),
                      L->s->killers.data(), L->s->countermoves.data(), L->stm, L->ply_init, L->depth,
                      L->max_nodes, L->s->tt1_entries, L->s->tt2_entries, L->finito);
}
}  // namespace

/* One cl_run_alphabeta launch (clrun.c:675-974): `workers` work-groups,
 * each on its own OS thread.  hash_history holds the game's hashes
 * (MAXGAMEPLY entries, copied per worker as search.c:55-64 does);
 * rnumbers holds 64 u32 per worker.  pv gets PV[64], counters 64 u64 per
 * worker. */
void ref_search_run(void *h, const uint64_t board[7], int stm, int depth, int ply_init,
                    const uint64_t *hash_history, const uint32_t *rnumbers, uint64_t max_nodes,
                    uint32_t *pv, uint64_t *counters) {
  RefSearch *s = (RefSearch *)h;
  int W = s->workers;
  std::vector<unsigned long> cnt((size_t)W * 64, 0), mv1((size_t)W * kMaxPly * 64, 0),
      mv2((size_t)W * kMaxPly * 64, 0), hist((size_t)W * kMaxGamePly, 0);
  std::vector<unsigned int> rn((size_t)W * 64, 0), pvbuf(kMaxPly, 0);
  for (int w = 0; w < W; w++) {
    if (hash_history) memcpy(&hist[(size_t)w * kMaxGamePly], hash_history, kMaxGamePly * sizeof(uint64_t));
    if (rnumbers) memcpy(&rn[(size_t)w * 64], rnumbers + (size_t)w * 64, 64 * sizeof(uint32_t));
  }
  unsigned int finito = 0;
  std::vector<std::thread> pool;
  std::vector<SearchLaunch> L(W);
  for (int w = 0; w < W; w++) {
    L[w] = SearchLaunch{s, board, &cnt, rn.data(), pvbuf.data(), &mv1, &mv2, &hist, &finito,
                        stm, ply_init, depth, max_nodes, w};
  }
  auto run = [&](int w) {
    /* gid = id0*size1 + id1 with a (workers, 1, 64) launch */
    refshim::set_work_item((unsigned long)w, 0, (unsigned long)W, 1);
    refshim::run_workgroup(search_body, &L[w], 64);
  };
  if (W == 1) run(0);
  else {
    for (int w = 0; w < W; w++) pool.emplace_back(run, w);
    for (auto &t : pool) t.join();
  }
  if (pv) memcpy(pv, pvbuf.data(), kMaxPly * sizeof(uint32_t));
  if (counters) memcpy(counters, cnt.data(), (size_t)W * 64 * sizeof(uint64_t));
}

int ref_tte_size(void) { return refshim_tte_size(); }

}  // extern "C"
