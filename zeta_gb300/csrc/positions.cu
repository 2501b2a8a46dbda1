/*
 * positions.cu -- seeded synthetic positions, generated on the device.
 *
 * The benchmark workloads are random legal playouts from the initial
 * position.  Position i of a batch is a pure function of (seed, i):
 *
 *   s = seed ^ (0xD1B54A32D192ED03 * (i + 1))         splitmix64 state
 *   repeat (at most 64 attempts):
 *     plies = min_plies + next(s) % (max_plies - min_plies + 1)
 *     play `plies` moves, each moves[next(s) % n] from the legal moves
 *       sorted by (from, to)
 *     accept if the side to move still has a legal move and at least
 *       min_pieces pieces remain
 *   depth = min_depth + next(s) % (max_depth - min_depth + 1)
 *
 * The oracle implements the same definition (zo_make_position) so tests
 * can compare the two.  The board carries a full Zobrist hash and the
 * half-move clock, like a board set by setboard (src/io.c:335-531).
 */
#include "context.cuh"
#include "tables.cuh"

namespace zeta {

ZHD u64 splitmix_next(u64 &s) {
  u64 z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ __forceinline__ int move_key(Move m) { return (m_from(m) << 6) | m_to(m); }

/* k-th legal move in (from, to) order, without sorting the list */
__device__ Move kth_sorted(const Move *list, int n, int k) {
  /* selection by rank: the move whose key has exactly k smaller keys */
  for (int i = 0; i < n; i++) {
    int key = move_key(list[i]), rank = 0;
    for (int j = 0; j < n; j++) rank += move_key(list[j]) < key;
    if (rank == k) return list[i];
  }
  return list[0];
}

__global__ void k_positions(u64 seed, int n, int min_plies, int max_plies, int min_pieces, int min_depth,
                            int max_depth, uint64_t *boards, uint8_t *stm_out, uint8_t *depth_out,
                            uint32_t *failures) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  u64 s = seed ^ (0xD1B54A32D192ED03ULL * (u64)(i + 1));
  Move list[256];
  for (int attempt = 0; attempt < 64; attempt++) {
    int plies = min_plies + (int)(splitmix_next(s) % (u64)(max_plies - min_plies + 1));
    Pos p = start_pos();
    int stm = 0, hmc = 0;
    bool ok = true;
    for (int k = 0; k < plies && ok; k++) {
      int nm = gen_legal(p, stm, false, list);
      if (nm == 0) {
        ok = false;
        break;
      }
      Move m = kth_sorted(list, nm, (int)(splitmix_next(s) % (u64)nm));
      hmc = next_hmc(hmc, m);
      play(p, m, false);
      stm ^= 1;
    }
    if (!ok || count_legal(p, stm) == 0 || popc(p.p1 | p.p2 | p.p3) < min_pieces) continue;
    uint64_t *b = boards + 7 * (size_t)i;
    b[0] = p.b0;
    b[1] = p.p1;
    b[2] = p.p2;
    b[3] = p.p3;
    b[4] = p.cr;
    b[5] = compute_hash(p, stm);
    b[6] = (uint64_t)hmc;
    stm_out[i] = (uint8_t)stm;
    depth_out[i] = (uint8_t)(min_depth + (int)(splitmix_next(s) % (u64)(max_depth - min_depth + 1)));
    return;
  }
  atomicAdd(failures, 1u);
  depth_out[i] = 0;
}

int positions_launch(u64 seed, int n, int min_plies, int max_plies, int min_pieces, int min_depth, int max_depth,
                     uint64_t *d_boards, uint8_t *d_stm, uint8_t *d_depth, uint32_t *d_fail, cudaStream_t s) {
  ZCHECK(cudaMemsetAsync(d_fail, 0, sizeof(uint32_t), s));
  k_positions<<<(n + 63) / 64, 64, 0, s>>>(seed, n, min_plies, max_plies, min_pieces, min_depth, max_depth,
                                           d_boards, d_stm, d_depth, d_fail);
  ZCHECK(cudaGetLastError());
  return ZETA_OK;
}

}  // namespace zeta
