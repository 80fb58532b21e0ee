"""CPU model of the persistent request server's work queue
(tiny_mc_gb300/csrc/tmc_serve.cu: publish_queue, harvest_queue;
tiny_mc_gb300/csrc/tmc_batch.cuh: queue_try_claim, publish_item_at).

Items live in a pool of P slots, freed as each item finishes (in any order);
the queue is a ring of 2P slot numbers in publishing order.  The host keeps at
most P items published and unfinished, writes a position's slot number
before it advances the published count, and frees a slot only when it reads
the item's completion.  A block reads the next position's slot number first
and then claims the position with a compare-and-swap on the claim counter;
the read is valid when the swap succeeds, because the host rewrites that
entry 2P positions later, only after P more items claimed after it have
finished.  Completions go to a ring of P entries in finishing order.

Every step below is one indivisible operation, interleaved at random (blocks
at different speeds, so one can stall between two of its steps) with a small
pool so that the rings wrap many times.  The model checks that every
successful claim read the slot published at its position, that no slot is
held by two unfinished items, and that the completion ring never overwrites
an unread entry.  Reading the entry after the swap instead of before fails
these checks under some of the same schedules."""
import random

import pytest


def run(seed, P, n_items, n_blocks):
    rng = random.Random(seed)
    Q = 2 * P
    order = [None] * Q                  # (position, slot) as written
    published = 0                       # host: positions published
    counter = 0                         # device: positions claimed
    free = list(range(P))
    slot_item = {}                      # slot -> item (position) holding it
    ring = [None] * P                   # completion ring entries
    done_tail = 0                       # device: completions appended
    done_head = 0                       # host: completions read
    next_item = 0
    blocks = [{"state": "idle"} for _ in range(n_blocks)]
    # blocks run at different speeds, so that one can stall between two of
    # its steps while the others finish many items
    weights = [0.4, 0.4] + [rng.choice([0.01, 0.2, 1.0]) for _ in range(n_blocks)]
    finished = 0
    steps = 0
    while finished < n_items:
        steps += 1
        assert steps < 2000000, "no progress"
        actors = ["host_publish", "host_harvest"] + list(range(n_blocks))
        a = rng.choices(actors, weights)[0]
        if a == "host_publish":
            outstanding = published - done_head
            if next_item < n_items and free and outstanding < P:
                slot = free.pop(rng.randrange(len(free)))   # any free slot
                assert slot not in slot_item
                slot_item[slot] = published
                order[published % Q] = (published, slot)
                published += 1                               # release store
                next_item += 1
        elif a == "host_harvest":
            e = ring[done_head % P]
            if e is not None:                                # ready flag set
                pos, slot = e
                assert slot_item.get(slot) == pos
                del slot_item[slot]
                free.append(slot)
                ring[done_head % P] = None
                done_head += 1
                finished += 1
        else:
            b = blocks[a]
            if b["state"] == "idle":                         # read counter, then entry
                c = counter
                if c < published:
                    b.update(state="read", c=c, entry=order[c % Q])
            elif b["state"] == "read":                       # compare-and-swap
                if counter == b["c"]:
                    counter += 1
                    pos, slot = b["entry"]
                    assert pos == b["c"], "claimed an entry overwritten before its claim"
                    assert slot_item.get(slot) == pos
                    b.update(state="walk", pos=pos, slot=slot)
                else:
                    b["state"] = "idle"                      # lost the race: retry
            elif b["state"] == "walk":                       # finish: append completion
                t = done_tail
                done_tail += 1
                assert ring[t % P] is None, "completion ring overran an unread entry"
                ring[t % P] = (b["pos"], b["slot"])
                b["state"] = "idle"
    assert counter == published == n_items == done_head
    assert not slot_item and sorted(free) == list(range(P))


@pytest.mark.parametrize("seed", range(60))
def test_queue_positions_carry_slots(seed):
    rng = random.Random(1000 + seed)
    run(seed, P=rng.choice([1, 2, 3, 4, 8]), n_items=rng.randint(50, 400), n_blocks=rng.randint(2, 6))
