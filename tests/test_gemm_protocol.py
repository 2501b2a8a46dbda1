"""The barrier protocol of the persistent tensor-core GEMM
(k_gemm_persist, zeta_gb300/csrc/mlp.cu), restated as a model and run
with random latencies on the CPU: a producer that fills a ring of K-slice
slots across tiles, an MMA issuer that writes tile j into accumulator
j & 1, four epilogue warps that drain an accumulator and release it.  Each
wait in the kernel is a parity wait on an mbarrier; the model checks that
when the kernel waits for completion k of a barrier, that barrier has
completed at most k + 1 phases (so the parity is unambiguous), that no
role waits forever, that an accumulator is read only after its tile's
MMAs and refilled only after all four warps released it, and that every
tile is stored once."""
import random

import pytest


class Bar:
    """An mbarrier: `count` arrivals complete a phase."""

    def __init__(self, count):
        self.count, self.arrived, self.done = count, 0, 0

    def arrive(self):
        self.arrived += 1
        if self.arrived == self.count:
            self.arrived, self.done = 0, self.done + 1


def simulate(ntiles, nkb, stages, seed):
    rnd = random.Random(seed)
    full = [Bar(1) for _ in range(stages)]
    empty = [Bar(1) for _ in range(stages)]
    acc_full, acc_empty = [Bar(1), Bar(1)], [Bar(4), Bar(4)]
    pending, now = [], [0]
    state, owner, reads = ["free", "free"], [None, None], [0] * ntiles

    def later(dt, fn):
        pending.append((now[0] + dt, fn))

    def ready(bar, k):
        assert bar.done <= k + 1, "parity wait would be ambiguous"
        return bar.done >= k + 1

    def producer():
        it = 0
        for _ in range(ntiles):
            for _ in range(nkb):
                slot, use = it % stages, it // stages
                while use > 0 and not ready(empty[slot], use - 1):
                    yield
                later(rnd.randint(1, 30), full[slot].arrive)  # the TMA copy lands
                it += 1

    def issuer():
        it = 0
        for j in range(ntiles):
            a = j & 1
            while j >= 2 and not ready(acc_empty[a], (j >> 1) - 1):
                yield
            assert state[a] == "free"
            state[a], owner[a] = "mma", j
            for _ in range(nkb):
                slot = it % stages
                while not ready(full[slot], it // stages):
                    yield
                later(rnd.randint(1, 10), empty[slot].arrive)  # commit: MMAs done reading the slot
                it += 1

            def finished(a=a, j=j):
                assert owner[a] == j
                state[a] = "ready"
                acc_full[a].arrive()
            later(rnd.randint(1, 10), finished)

    def epilogue_warp():
        for j in range(ntiles):
            a = j & 1
            while not ready(acc_full[a], j >> 1):
                yield
            assert owner[a] == j and state[a] in ("ready", "reading")
            state[a] = "reading"
            for _ in range(rnd.randint(0, 20)):
                yield
            reads[j] += 1
            if reads[j] == 4:
                state[a] = "free"
            acc_empty[a].arrive()

    roles = [producer(), issuer()] + [epilogue_warp() for _ in range(4)]
    steps = 0
    while roles or pending:
        steps += 1
        assert steps < 10 ** 6, "a role waits forever"
        now[0] += 1
        for p in [p for p in pending if p[0] <= now[0]]:
            pending.remove(p)
            p[1]()
        for r in list(roles):
            try:
                next(r)
            except StopIteration:
                roles.remove(r)
    assert reads == [4] * ntiles


@pytest.mark.parametrize("stages", [2, 4, 6, 8])
def test_persistent_gemm_barrier_protocol(stages):
    for ntiles in (1, 2, 3, 7):
        for nkb in (1, 2, 4, 12):
            for seed in range(6):
                simulate(ntiles, nkb, stages, seed)
