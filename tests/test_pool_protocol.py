"""A model check of the block pool's protocol (persistent.cuh: pool_exchange,
sample_loop, drain_loop) on the host: warps of one block run chunks of their
samples, refill from a list (fixed, or filled by producers over time), and
trade samples through the pool under its lock, in seeded random orders.  The
rules are the kernel's; the check is that every sample finishes exactly once,
that no sample is left in the pool when the last warp leaves, and that warps
end up carrying fuller lanes than without the pool."""
import random

import pytest

LANES, COMPACT_BELOW, CAP = 32, 16, 128


class Block:
    def __init__(self, warps, lengths, produced_at, use_pool, rng):
        self.rng = rng
        self.len = dict(enumerate(lengths))
        self.produced_at = produced_at  # sample -> tick at which it enters the list
        self.queue = []
        self.pending = sorted(self.len, key=lambda s: produced_at[s])
        self.pool = []
        self.alive = 0
        self.held_all = 0
        self.use_pool = use_pool
        self.done = []
        self.warps = [dict(lanes={}, held=0, left=False, entered=False) for _ in range(warps)]
        self.lane_slots = 0  # warp-chunks run, times 32
        self.lane_work = 0   # sample-chunks run

    def produce(self, tick):
        while self.pending and self.produced_at[self.pending[0]] <= tick:
            self.queue.append(self.pending.pop(0))

    def closed(self):
        return not self.pending and not self.queue

    def exchange(self, w, closed):
        lanes = w["lanes"]
        count, k = len(self.pool), len(lanes)
        leave = False
        if 0 < k < COMPACT_BELOW and count + k <= CAP and (
                not closed or (self.alive - 1) * LANES >= self.held_all - w["held"] + k + count):
            self.pool.extend(lanes.items())
            lanes.clear()
            count, k = len(self.pool), 0
            leave = closed
        if not leave:
            idle = LANES - k
            if idle > 0 and count > 0 and (k >= COMPACT_BELOW or closed or count >= COMPACT_BELOW):
                take = min(idle, count)
                for _ in range(take):
                    s, rem = self.pool.pop()
                    lanes[s] = rem
                k += take
            if k == 0 and closed and not self.pool:
                leave = True
        self.held_all += (0 if leave else k) - w["held"]
        if leave:
            self.alive -= 1
        w["held"] = 0 if leave else k
        return leave

    def step(self, w, chunk):
        """One iteration of the warp's loop; False when the warp has left."""
        if not w["entered"]:
            w["entered"] = True
            self.alive += 1
        lanes = w["lanes"]
        need = LANES - len(lanes)
        dry = False
        if need:
            got = self.queue[:need]
            del self.queue[:need]
            for s in got:
                lanes[s] = self.len[s]
            dry = len(got) < need
        closed = self.closed()
        if self.use_pool and (dry or closed) and self.exchange(w, closed):
            w["left"] = True
            return False
        if not lanes:
            if self.use_pool:
                return True  # parked: waits for samples
            if closed:
                w["left"] = True
                self.alive -= 1
                return False
            return True
        self.lane_slots += LANES
        self.lane_work += len(lanes)
        for s in list(lanes):
            lanes[s] -= chunk
            if lanes[s] <= 0:
                del lanes[s]
                self.done.append(s)
        return True


def run(seed, use_pool, producers):
    rng = random.Random(seed)
    n = rng.randint(100, 700)
    lengths = [rng.choice([rng.randint(1, 40), rng.randint(40, 400), rng.randint(400, 4000)])
               for _ in range(n)]
    produced_at = {s: (rng.randint(0, 3000) if producers else 0) for s in range(n)}
    b = Block(rng.choice([2, 4, 8]), lengths, produced_at, use_pool, rng)
    tick = 0
    live = list(range(len(b.warps)))
    while live:
        tick += 1
        assert tick < 10 ** 6, "no progress"
        b.produce(tick)
        w = b.warps[rng.choice(live)]
        if not b.step(w, chunk=32):
            live = [i for i in live if not b.warps[i]["left"]]
    return b


@pytest.mark.parametrize("producers", [False, True], ids=["fixed-list", "drained-list"])
def test_every_sample_once_and_nothing_stranded(producers):
    for seed in range(60):
        b = run(seed, use_pool=True, producers=producers)
        assert sorted(b.done) == sorted(b.len), seed  # every sample exactly once
        assert not b.pool and not b.queue and not b.pending
        assert b.alive == 0 and b.held_all == 0


def test_pool_keeps_lanes_fuller():
    with_pool = without = 0.0
    for seed in range(30):
        a = run(seed, use_pool=True, producers=False)
        c = run(seed, use_pool=False, producers=False)
        assert sorted(c.done) == sorted(c.len)
        with_pool += a.lane_work / a.lane_slots
        without += c.lane_work / c.lane_slots
    assert with_pool > without
