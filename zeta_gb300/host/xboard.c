/*
 * xboard.c -- the command loop of the zeta host (src/xboard.c:44-1499):
 * the CECP/xboard commands a GUI uses to play, plus the console commands
 * `perft` and `selftest`.  Unknown commands are answered with
 * "Error (unknown command)" as CECP asks.
 */
#include <inttypes.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/clrun.h"
#include "../../include/zeta_cuda.h"
#include "engine.h"

static bool xboard_mode = false, force_mode = false, post = true;

static void new_game(void) {
  int full;
  board_setfen(BOARD, &STM, &full, "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1");
  PLY = 0;
  GAMEPLY = 0;
  memset(HashHistory, 0, sizeof HashHistory);
  HashHistory[0] = BOARD[QBBHASH];
  /* a new game starts from an empty table (src/xboard.c:159-199) */
  if (!cl_release_device() || !cl_init_device("alphabeta_gpu")) exit(EXIT_FAILURE);
}

static void play_move(Move m) {
  board_play(BOARD, STM, m);
  STM = !STM;
  PLY++;
  GAMEPLY++;
  if (PLY < MAXGAMEPLY) {
    HashHistory[PLY] = BOARD[QBBHASH];
    MoveHistory[PLY] = m;
  }
}

/* The legal move a user's move text names, or 0.  The text must be
 * coordinate notation (move_text_ok); the position's legal moves come from
 * the device's perft generator with all four promotions, and a promotion
 * without a piece letter is taken as the queen's.  The reference plays
 * whatever the text decodes to (src/xboard.c, usermove). */
static Move legal_user_move(const char *mvs) {
  if (!move_text_ok(mvs)) return 0;
  const Move m = can2move(mvs, BOARD, STM);
  uint32_t list[256];
  int32_t n = 0;
  const uint8_t side = (uint8_t)STM;
  if (zeta_genmoves_batch(BOARD, &side, 1, 8, list, &n) != ZETA_OK) {
    printf("Error (device): %s\n", zeta_last_error());
    return 0;
  }
  for (int i = 0; i < n; i++) {
    const Move g = list[i];
    if (GETSQFROM(g) != GETSQFROM(m) || GETSQTO(g) != GETSQTO(m)) continue;
    const int kind = GETPTO(g) >> 1, asked = GETPTO(m) >> 1;
    if ((GETPFROM(g) >> 1) != PAWN || kind == PAWN) return g; /* not a promotion */
    if (asked == kind || (asked == PAWN && kind == QUEEN)) return g;
  }
  return 0;
}

/* the node budget of a move from its time (src/xboard.c:193, 371) */
static void set_max_nodes(void) { MaxNodes = (uint64_t)(MaxTime / 1000 * (double)nodes_per_second); }

/* moves left in this session (one move kept as spare), src/xboard.c:358-359 */
static void update_moves_left(void) {
  if (timemode == 1 && MaxMoves > 0) MovesLeft = (MaxMoves - (((PLY + 1) / 2) % MaxMoves)) + 1;
}

static void think_and_move(void) {
  const double t0 = get_time_ms();
  Move m = rootsearch(BOARD, STM, SD);
  if (JUSTMOVE(m) == MOVENONE) {
    printf("resign\n");
    return;
  }
  char mv[6];
  move2can(m, mv);
  play_move(m);
  printf("move %s\n", mv);
  fflush(stdout);
  /* clock after the move, src/xboard.c:355-371 */
  TimeLeft -= get_time_ms() - t0;
  update_moves_left();
  if (timemode == 0) TimeLeft = TimeBase;
  if (timemode == 2) TimeLeft += TimeInc;
  MaxTime = TimeLeft / (MovesLeft > 0 ? MovesLeft : 1) + TimeInc;
  if (timemode == 1 && MovesLeft == 2) TimeLeft += TimeBase;
  set_max_nodes();
}

void xboard(void) {
  char line[4096];
  new_game();
  while (fgets(line, sizeof line, stdin)) {
    char cmd[64] = {0};
    if (sscanf(line, "%63s", cmd) != 1) continue;
    const char *arg = line + strlen(cmd);
    while (*arg == ' ') arg++;
    if (LogFile) fprintf(LogFile, "> %s", line);
    if (!strcmp(cmd, "xboard")) {
      xboard_mode = true;
      printf("\n");
    } else if (!strcmp(cmd, "protover")) {
      printf("feature done=0\nfeature myname=\"Zeta GB300\" ping=1 setboard=1 usermove=1 sigint=0 sigterm=0\n"
             "feature colors=0 analyze=0 memory=0 reuse=1\nfeature done=1\n");
    } else if (!strcmp(cmd, "new")) {
      new_game();
      force_mode = false;
      SD = MAXPLY - 1;
      set_max_nodes();
    } else if (!strcmp(cmd, "setboard")) {
      int full;
      if (!board_setfen(BOARD, &STM, &full, arg)) printf("tellusererror Illegal position\n");
      PLY = 0;
      HashHistory[0] = BOARD[QBBHASH];
    } else if (!strcmp(cmd, "force")) {
      force_mode = true;
    } else if (!strcmp(cmd, "go")) {
      force_mode = false;
      think_and_move();
    } else if (!strcmp(cmd, "usermove")) {
      char mvs[16] = {0};
      sscanf(arg, "%15s", mvs);
      const Move m = legal_user_move(mvs);
      if (!m) {
        printf("Illegal move: %s\n", mvs);
        continue;
      }
      play_move(m);
      if (!force_mode) think_and_move();
    } else if (!strcmp(cmd, "sd")) {
      SD = atoi(arg);
      if (SD < 1) SD = 1;
      if (SD >= MAXPLY) SD = MAXPLY - 1;
    } else if (!strcmp(cmd, "level")) {
      /* level MPS BASE INC, BASE in minutes or min:sec (src/xboard.c:384-424) */
      int mps = 0, min = 0, sec = 0;
      double inc = 0;
      if (sscanf(arg, "%d %d:%d %lf", &mps, &min, &sec, &inc) != 4 &&
          sscanf(arg, "%d %d %lf", &mps, &min, &inc) != 3)
        continue;
      if (strchr(arg, ':') == NULL) sec = 0;
      MaxMoves = mps;
      TimeBase = (60.0 * min + sec) * 1000;
      TimeInc = inc * 1000;
      TimeLeft = TimeBase;
      timemode = MaxMoves == 0 ? 2 : 1;
      MovesLeft = timemode == 2 ? 40 : 1;
      update_moves_left();
      MaxTime = TimeLeft / MovesLeft + TimeInc;
      set_max_nodes();
    } else if (!strcmp(cmd, "st")) {
      /* st SECONDS: a fixed time per move (src/xboard.c:426-438) */
      double secs = 0;
      if (sscanf(arg, "%lf", &secs) != 1 || secs <= 0) continue;
      TimeBase = TimeLeft = secs * 1000;
      TimeInc = 0;
      MovesLeft = MaxMoves = 1;
      timemode = 0;
      MaxTime = TimeLeft / MovesLeft + TimeInc;
      set_max_nodes();
    } else if (!strcmp(cmd, "time")) {
      /* time CENTISECONDS left on the engine's clock (src/xboard.c:440-453) */
      double cs = 0;
      if (sscanf(arg, "%lf", &cs) != 1) continue;
      TimeLeft = cs * 10;
      update_moves_left();
      MaxTime = TimeLeft / (MovesLeft > 0 ? MovesLeft : 1) + TimeInc;
      set_max_nodes();
    } else if (!strcmp(cmd, "otim")) {
      /* the opponent's clock: not used (src/xboard.c:455-456) */
    } else if (!strcmp(cmd, "ping")) {
      printf("pong %s", arg);
    } else if (!strcmp(cmd, "post")) {
      post = true;
    } else if (!strcmp(cmd, "nopost")) {
      post = false;
    } else if (!strcmp(cmd, "quit")) {
      break;
    } else if (!strcmp(cmd, "perft") && !xboard_mode) {
      int depth = atoi(arg);
      if (depth < 1) depth = SD < 16 ? SD : 6;
      printf("### computing perft depth %d: ###\n", depth);
      if (!cl_release_device() || !cl_init_device("perft_gpu")) exit(EXIT_FAILURE);
      double t0 = get_time_ms();
      perft(BOARD, STM, depth);
      double s = (get_time_ms() - t0 + 1) / 1000.0;
      printf("nodecount:%" PRIu64 ", seconds: %lf, nps: %" PRIu64 " \n", ABNODECOUNT, s, (uint64_t)(ABNODECOUNT / s));
      if (!cl_release_device() || !cl_init_device("alphabeta_gpu")) exit(EXIT_FAILURE);
    } else if (!strcmp(cmd, "promotions") && !xboard_mode) {
      /* promotions all|queen: the promotion rule of the perft command
       * (queen only is the reference's, and the default) */
      char rule[16] = {0};
      sscanf(arg, "%15s", rule);
      if (!strcmp(rule, "all")) cl_set_all_promotions(1);
      else if (!strcmp(rule, "queen")) cl_set_all_promotions(0);
      else printf("Error (usage: promotions all|queen)\n");
    } else if (!strcmp(cmd, "selftest") && !xboard_mode) {
      selftest();
    } else if (!strcmp(cmd, "benchsmp") && !xboard_mode) {
      /* benchsmp [max workers]: worker scaling of the search to depth sd */
      uint64_t maxw = strtoull(arg, NULL, 10);
      benchsmp(BOARD, STM, SD, maxw ? maxw : totalWorkUnits);
    } else if (!strcmp(cmd, "benchfile") && !xboard_mode) {
      /* benchfile <file of FEN lines> [max workers]: benchsmp on every
       * position, then the summed table (benchkaufmann / benchhyatt24) */
      char path[512] = {0};
      unsigned long long maxw = 0;
      if (sscanf(arg, "%511s %llu", path, &maxw) < 1) {
        printf("Error (usage: benchfile <file> [max workers])\n");
      } else {
        benchfile(path, SD, maxw ? (uint64_t)maxw : totalWorkUnits);
        HashHistory[0] = BOARD[QBBHASH];
      }
    } else if (!strcmp(cmd, "print") && !xboard_mode) {
      char fen[256];
      board_print(BOARD, STM);
      board_getfen(BOARD, STM, 1 + PLY / 2, fen, sizeof fen);
      printf("# %s\n", fen);
    } else if (!strcmp(cmd, "help") && !xboard_mode) {
      printf("# commands: new, setboard <fen>, go, usermove <move>, force, sd <depth>, st <seconds>,\n"
             "# level <moves> <minutes> <increment>, time <centiseconds>, perft <depth>,\n"
             "# promotions all|queen (perft's promotion rule),\n"
             "# benchfile <file of FENs> [max workers],\n"
             "# benchsmp [max workers], selftest, print, quit (and the xboard protocol)\n");
    } else if (!strcmp(cmd, "accepted") || !strcmp(cmd, "rejected") || !strcmp(cmd, "random") ||
               !strcmp(cmd, "computer") || !strcmp(cmd, "result") || !strcmp(cmd, "hard") ||
               !strcmp(cmd, "easy") || !strcmp(cmd, "name") || !strcmp(cmd, "rating") || !strcmp(cmd, "white") ||
               !strcmp(cmd, "black") || !strcmp(cmd, "draw") || !strcmp(cmd, "memory")) {
      /* accepted and ignored */
    } else {
      printf("Error (unknown command): %s\n", cmd);
    }
    (void)post;
    fflush(stdout);
  }
}
