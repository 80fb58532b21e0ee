"""CPU model of the shared-histogram tallies of the walk kernels
(tiny_mc_gb300/csrc/tmc_walk.cuh: tally_add_nowrap, swap_flush_tally,
flush_steps), which replace the float += of photon.c:30-31.

A block's lanes deposit 41-bit fixed-point values into a 64-bit sum kept as
two 32-bit shared words (low word by an atomic add whose old value gives the
carry, then the high word with that carry), while any warp may take both
words with atomic exchanges against zero and add them into the 128-bit global
tally.  Each atomic step is modelled as one indivisible operation and the
steps of the depositing lanes and of a flushing warp are interleaved at
random: the global tally plus what is left must equal the exact sum of the
deposits, and the per-item probe (the flushed w sums of one shell plus the
remainder) must equal that shell's exact sum."""
import random

import pytest

M32 = (1 << 32) - 1


def split_fx40(v):
    """The (lo, hi) words of a deposit of v < 2^41 fixed-point units."""
    return v & M32, v >> 32


def run_schedule(rng, n_lanes, deposits_per_lane, n_flushes):
    lo = hi = 0                 # the shared words of one shell
    glob = 0                    # the 128-bit global tally
    probe_acc, probe_hi = 0, 0  # 64-bit shared accumulator + its wraps
    want = 0
    # each lane: a list of pending atomic steps; a deposit is two steps
    lanes = []
    for _ in range(n_lanes):
        steps = []
        for _ in range(deposits_per_lane):
            v = rng.randrange(0, 1 << 41) if rng.random() < 0.5 else rng.choice([0, 1, M32, 1 << 40])
            want += v
            steps.append(("lo", v))
        lanes.append(steps)
    lane_state = [None] * n_lanes       # carry-in pending for the hi step
    flusher = []                        # pending steps of flushes
    for _ in range(n_flushes):
        flusher += [("xlo",), ("xhi",), ("add",)]
    taken = {}
    while any(lanes) or any(s is not None for s in lane_state) or flusher:
        choices = [i for i in range(n_lanes) if lanes[i] or lane_state[i] is not None]
        if flusher:
            choices.append(-1)
        who = rng.choice(choices)
        if who == -1:
            op = flusher.pop(0)
            if op[0] == "xlo":
                taken["lo"], lo = lo, 0
            elif op[0] == "xhi":
                taken["hi"], hi = hi, 0
            else:
                v = (taken.pop("hi") << 32) | taken.pop("lo")
                glob += v
                old = probe_acc
                probe_acc = (probe_acc + v) & ((1 << 64) - 1)
                probe_hi += 1 if probe_acc < old else 0
            continue
        if lane_state[who] is not None:          # second step: the high word
            add = lane_state[who]
            assert hi + add <= M32, "high word overflow: the flush bound is broken"
            hi += add
            lane_state[who] = None
            continue
        _, v = lanes[who].pop(0)                 # first step: the low word
        v_lo, v_hi = split_fx40(v)
        old = lo
        lo = (lo + v_lo) & M32
        carry = 1 if ((old + v_lo) & M32) < old else 0
        lane_state[who] = v_hi + carry
    rest = (hi << 32) | lo
    total = glob + rest
    probe = (probe_hi << 64) + probe_acc + rest
    return want, total, probe


@pytest.mark.parametrize("seed", range(40))
def test_exchange_flush_keeps_sums_exact(seed):
    rng = random.Random(seed)
    want, total, probe = run_schedule(rng, n_lanes=rng.randint(1, 8),
                                      deposits_per_lane=rng.randint(1, 40),
                                      n_flushes=rng.randint(0, 12))
    assert total == want
    assert probe == want


def test_high_word_bound_per_flush_interval():
    """flush_steps(lanes) = 2^23 / lanes: with every lane checked at every
    multiple it reaches, a lane deposits at most flush_steps + 1 times between
    two flushes, each deposit adding at most 2^8 + 1 to a high word."""
    for lanes in (32, 128, 256, 512):
        flush_steps = (1 << 23) // lanes
        assert lanes * (2 ** 8 + 1) * (flush_steps + 1) < 2 ** 32
    # and a deposit of w <= 1 has hi = floor(w * 2^8) <= 2^8
    assert split_fx40(1 << 40)[1] == 1 << 8
