/*
 * main.c -- the zeta host binary (src/zeta.c:525-709): options, config,
 * device start-up, then the xboard command loop.
 *
 *   zeta [-s|--selftest] [-l|--log] [-p|--pure] [-d <device>] [-c <config.txt>] [-v] [-h]
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
         "  -d <n>           CUDA device (default 0)\n"
         "  -c <file>        config file (default config.txt: threadsX, threadsY, tt1_memory, ...)\n"
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
      search_mode = 0;
    } else if (!strcmp(argv[i], "-l") || !strcmp(argv[i], "--log")) {
      LogFile = fopen("zeta.log", "a");
    } else if (!strcmp(argv[i], "-d") && i + 1 < argc) {
      dev = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "-c") && i + 1 < argc) {
      config = argv[++i];
    } else {
      usage();
      return 1;
    }
  }
  read_config(config);
  if (dev >= 0) device_id = dev;
  if (!engine_alloc()) {
    fprintf(stderr, "Error: out of host memory\n");
    return 1;
  }
  if (!cl_init_device("alphabeta_gpu")) return 1;
  int rc = 0;
  if (run_selftest) rc = selftest() == 14 ? 0 : 1;
  else xboard();
  cl_release_device();
  engine_free();
  if (LogFile) fclose(LogFile);
  return rc;
}
