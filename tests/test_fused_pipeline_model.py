"""CPU model of the warp-specialised inference kernel's hand-offs
(mlp_tc_fused_kernel in hairmsnn_gb300/csrc/hm_mlp_tc.cu), run under random
interleavings.

Actors, as in the kernel: NS encoder teams (team t writes the CTA's tiles
k = t (mod NS) into stage t) and two layer lanes (lane s reads the tiles
k = s (mod 2) from stage k % NS).  Barriers are mbarriers with one arrival
per phase; a parity wait passes once the phase of that parity has completed,
which includes "at once" for parity 1 before any phase completed, exactly
the rule the hardware applies to mbarrier.try_wait.parity.

  team t, its j-th tile k:   j > 0: wait empty[t] parity (j - 1) & 1
                             write stage t := k;  arrive full[t]
  lane s, tile k:            wait full[k % NS] parity (k / NS) & 1
                             read stage k % NS (must hold k);  arrive empty[k % NS]

With an even NS (the kernel's 6 or 2) every stage feeds one lane only and
every read sees its own tile in all schedules.  With an odd NS a lane can
wait on a stage for the second time before the other lane's first phase on
it has completed, and the parity wait passes early; the model finds such a
schedule, which is why the kernel uses only even stage counts.
"""
import random

import pytest


class MBar:
    def __init__(self):
        self.completed = 0  # phases completed (one arrival each)

    def arrive(self):
        self.completed += 1

    def passes(self, parity):
        # try_wait.parity: the current (incomplete) phase has parity
        # completed & 1; a wait for the other parity passes
        return (self.completed & 1) != parity


def run(ns, n_tiles, seed):
    rng = random.Random(seed)
    full = [MBar() for _ in range(ns)]
    empty = [MBar() for _ in range(ns)]
    stage = [None] * ns
    errors = []

    def team(t):
        j = 0
        for k in range(t, n_tiles, ns):
            if j > 0:
                while not empty[t].passes((j - 1) & 1):
                    yield
            yield  # the encoding itself takes time
            stage[t] = k
            full[t].arrive()
            j += 1

    def lane(s):
        for k in range(s, n_tiles, 2):
            st = k % ns
            while not full[st].passes((k // ns) & 1):
                yield
            if stage[st] != k:
                errors.append((s, k, stage[st]))
            yield  # the layer-0 MMAs read the stage: nobody may write it meanwhile
            if stage[st] != k:
                errors.append((s, k, stage[st]))
            empty[st].arrive()

    actors = [team(t) for t in range(ns)] + [lane(s) for s in range(2)]
    live = list(actors)
    steps = 0
    while live and not errors:  # a wrong read ends the run (the kernel's
        a = rng.choice(live)    # phases are out of step from there on)
        try:
            next(a)
        except StopIteration:
            live.remove(a)
        steps += 1
        assert steps < 10 ** 6, "no progress"
    return errors


@pytest.mark.parametrize("ns", [2, 6])
def test_even_stage_counts_hand_every_tile_to_its_lane(ns):
    for seed in range(300):
        for n_tiles in (1, 2, 3, ns, ns + 1, 2 * ns + 3, 40):
            assert run(ns, n_tiles, seed) == [], (ns, n_tiles, seed)


@pytest.mark.parametrize("ns", [1, 3])
def test_odd_stage_counts_let_a_parity_wait_pass_early(ns):
    found = any(run(ns, 12, seed) for seed in range(300))
    assert found
