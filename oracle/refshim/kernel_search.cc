/*
 * kernel_search.cc -- compiles the reference search kernel (src/zeta.cl,
 * unmodified, found on the include path) as host C++ under cl_shim.h.
 * TEST INFRASTRUCTURE ONLY (see kernel_perft.cc).
 */
#include "cl_shim.h"

namespace refsearch {
#include "zeta.cl"
}

/* one lane's entry into alphabeta_gpu (zeta.cl:852-873) */
extern "C" void refshim_search_lane(const unsigned long *board, unsigned long *counters,
                                    const unsigned int *rnumbers, unsigned int *pv,
                                    unsigned long *moves1, unsigned long *moves2,
                                    unsigned long *history, const unsigned long *between,
                                    const unsigned long *line, void *tt1, void *tt2,
                                    unsigned int *killers, unsigned int *countermoves, int stm,
                                    int ply_init, int depth, unsigned long max_nodes,
                                    unsigned long tt1_entries, unsigned long tt2_entries,
                                    unsigned int *finito) {
  refsearch::alphabeta_gpu(board, counters, rnumbers, pv, moves1, moves2, history, between, line,
                           (refsearch::TTE *)tt1, (refsearch::ABDADATTE *)tt2, killers, countermoves,
                           stm, ply_init, depth, max_nodes, tt1_entries, tt2_entries, finito);
}

/* sizes of the table entries as this compiler lays them out */
extern "C" int refshim_tte_size(void) { return (int)sizeof(refsearch::TTE); }
extern "C" int refshim_abdadatte_size(void) { return (int)sizeof(refsearch::ABDADATTE); }
