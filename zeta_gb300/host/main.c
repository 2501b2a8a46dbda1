/*
 * main.c -- the zeta host binary (src/zeta.c:525-709): options, config,
 * device start-up, then the xboard command loop.
 *
 *   zeta [-s|--selftest] [-l|--log] [-p|--pure] [-u|--allpromotions] [-d <device>] [-c <config.txt>]
 *        [-v] [-h]
 */
#include <stdlib.h>
#include <string.h>

#include "../../include/clrun.h"
#include "engine.h"

static void usage(void) {
  printf("Zeta GB300 -- the Zeta chess engine's device path on Blackwell GPUs.\n"
         "  -s, --selftest   run the 14 perft known-answer tests and exit\n"
         "  -l, --log        append a log to zeta.log\n"
         "  -p, --pure       pure fixed-depth alpha-beta (root score = negamax) instead of\n"
         "                   the reference's search with its heuristics\n"
         "  -u, --allpromotions  perft promotes to queen, rook, bishop or knight (the\n"
         "                   reference, and the default, promotes to a queen only)\n"
         "  -d <n>           CUDA device (default 0)\n"
         "  -c <file>        config file (default config.txt: threadsX, threadsY, tt1_memory, ...)\n"
         "  --guessconfig    measure the search on the device, write config.txt and exit\n"
         "  --guessconfigx   the same, longer and with more worker counts\n"
         "  -pl, -dl         list the platform / the devices and exit\n"
         "  -v, --version    print the version\n"
         "  -h, --help       this text\n"
         "Without options it reads xboard / console commands from stdin.\n");
}

int main(int argc, char **argv) {
  setvbuf(stdout, NULL, _IONBF, 0);
  bool run_selftest = false;
  const char *config = "config.txt";
  int dev = -1;
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "-h") || !strcmp(argv[i], "--help")) {
      usage();
      return 0;
    } else if (!strcmp(argv[i], "-v") || !strcmp(argv[i], "--version")) {
      printf("Zeta GB300 099m\n");
      return 0;
    } else if (!strcmp(argv[i], "-s") || !strcmp(argv[i], "--selftest")) {
      run_selftest = true;
    } else if (!strcmp(argv[i], "-p") || !strcmp(argv[i], "--pure")) {
      cl_set_pure_search(1);
    } else if (!strcmp(argv[i], "-u") || !strcmp(argv[i], "--allpromotions")) {
      cl_set_all_promotions(1);
    } else if (!strcmp(argv[i], "-l") || !strcmp(argv[i], "--log")) {
      LogFile = fopen("zeta.log", "a");
    } else if (!strcmp(argv[i], "-d") && i + 1 < argc) {
      dev = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "-c") && i + 1 < argc) {
      config = argv[++i];
    } else if (!strcmp(argv[i], "--guessconfig") || !strcmp(argv[i], "--guessconfigx")) {
      /* src/zeta.c:612-627: tune, write config.txt, exit */
      return cl_guess_config(!strcmp(argv[i], "--guessconfigx")) ? 0 : 1;
    } else if (!strcmp(argv[i], "-pl")) {
      return cl_platform_list() ? 0 : 1;
    } else if (!strcmp(argv[i], "-dl")) {
      return cl_device_list() ? 0 : 1;
    } else {
      usage();
      return 1;
    }
  }
  read_config(config);
  if (dev >= 0) opencl_device_id = dev;
  if (!engine_alloc()) {
    fprintf(stderr, "Error: out of host memory\n");
    return 1;
  }
  if (!cl_init_device("alphabeta_gpu")) return 1;
  /* the initial position and the start-up warm-up launch, as
   * src/zeta.c:687-698 */
  int fullmove = 1;
  if (!board_setfen(BOARD, &STM, &fullmove, "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")) return 1;
  memcpy(GLOBAL_BOARD, BOARD, 7 * sizeof(Bitboard));
  HashHistory[0] = BOARD[QBBHASH];
  memcpy(GLOBAL_HASHHISTORY, HashHistory, sizeof HashHistory);
  if (!cl_run_alphabeta(STM, 0, 1)) return 1;
  int rc = 0;
  if (run_selftest) rc = selftest() == 14 ? 0 : 1;
  else xboard();
  cl_release_device();
  engine_free();
  if (LogFile) fclose(LogFile);
  return rc;
}
