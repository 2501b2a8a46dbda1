/*
 * kernel_perft.cc -- compiles the reference perft kernel (src/zetaperft.cl,
 * unmodified, found on the include path) as host C++ under cl_shim.h.
 * TEST INFRASTRUCTURE ONLY.  The oracle Makefile preprocesses this file
 * into oracle/_ref/ where the reference tree is present; the result has
 * no system headers and compiles on either host architecture.
 */
#include "cl_shim.h"

namespace refperft {
#include "zetaperft.cl"
}

/* one lane's entry into perft_gpu (zetaperft.cl:801-812) */
extern "C" void refshim_perft_lane(const unsigned long *board, unsigned long *counters,
                                   unsigned long *moves, unsigned long *history,
                                   const unsigned long *between, const unsigned long *line, int stm,
                                   int depth) {
  refperft::perft_gpu(board, counters, moves, history, between, line, stm, 0, depth, 0);
}
