"""A model of the level-completion word of the persistent peel, checked on CPU.

One 64-bit word per level packs the work units finished (high half: the
participants' scans and the queued tasks) with the tasks pushed (low half,
also the queue cursor); the level is complete when units == participants +
tasks.  A participant pushes tasks only during its scan, before it arrives;
a task pushes tasks only while it runs, before it is finished; a task is
claimed only after its push (the claimer reads the entry written after the
push).  Under those rules no snapshot of the word shows the equality while
work remains, and the last finish shows it.  The model runs random
interleavings of those atomic steps (each a single add on the word, as on the
device) and checks both properties after every step.
"""
import random

import pytest

HALF = 32
MASK = (1 << HALF) - 1


def run(parts: int, seed: int, max_children: int = 3, max_tasks: int = 200, finish_first: bool = False):
    rng = random.Random(seed)
    word = 0
    scanning = {p: rng.randint(0, 3) for p in range(parts)}   # pushes left in each scan
    queued = 0            # pushed, not yet claimed
    running = []          # claimed tasks: pushes left in each
    pushed_total = 0
    while True:
        units, tail = word >> HALF, word & MASK
        all_done = not scanning and queued == 0 and not running
        complete = units == parts + tail
        assert complete == all_done, (units, tail, scanning, queued, running)
        if all_done:
            return pushed_total
        moves = []
        for p, left in scanning.items():
            moves.append(("scan_push", p) if left and pushed_total < max_tasks else ("arrive", p))
        if queued:
            moves.append(("claim", None))
        for i, left in enumerate(running):
            moves.append(("task_push", i) if left and pushed_total < max_tasks else ("finish", i))
        kind, who = rng.choice(moves)
        if kind == "scan_push":
            n = rng.randint(1, 3)
            word += n                      # atomicAdd(units_tail, n): reserve queue slots
            queued += n
            pushed_total += n
            scanning[who] -= 1
        elif kind == "arrive":
            word += 1 << HALF              # atomicAdd(units_tail, 1 << 32)
            del scanning[who]
        elif kind == "claim":
            queued -= 1
            running.append(rng.randint(0, max_children))
        elif kind == "task_push":
            n = rng.randint(1, 2)
            word += n
            queued += n
            pushed_total += n
            running[who] -= 1
        else:                              # finish one task
            word += 1 << HALF
            running.pop(who)
            if finish_first and rng.random() < 0.5 and pushed_total < max_tasks:
                # a planted mistake: the task publishes its finish before its
                # last push, so a snapshot between the two shows the level done
                units, tail = word >> HALF, word & MASK
                assert units != parts + tail, "the level reads complete while a push is pending"
                word += 1
                queued += 1
                pushed_total += 1


@pytest.mark.parametrize("parts", [1, 2, 7, 40])
def test_completion_word_is_exact_under_random_interleavings(parts):
    pushed = 0
    for seed in range(25):
        pushed += run(parts, seed, max_children=seed % 4)   # shallow to capped task trees
    assert pushed > 0


def test_the_model_catches_a_finish_published_before_a_push():
    with pytest.raises(AssertionError):
        for seed in range(25):
            run(2, seed, max_children=0, finish_first=True)
